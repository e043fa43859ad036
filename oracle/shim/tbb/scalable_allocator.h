#pragma once
#include "_shim_common.h"
namespace tbb {
template <typename T>
class scalable_allocator {
public:
    typedef T value_type;
    typedef T *pointer;
    typedef const T *const_pointer;
    typedef T &reference;
    typedef const T &const_reference;
    typedef std::size_t size_type;
    typedef std::ptrdiff_t difference_type;
    template <typename U> struct rebind { typedef scalable_allocator<U> other; };
    scalable_allocator() {}
    template <typename U> scalable_allocator(const scalable_allocator<U> &) {}
    pointer allocate(size_type n, const void * = 0) {
        size_type bytes = ((n * sizeof(T) + 127) / 128) * 128;
        if (bytes == 0) bytes = 128;
        void *p = nullptr;
        if (posix_memalign(&p, 128, bytes) != 0) p = nullptr;
        if (!p) throw std::bad_alloc();
        return static_cast<pointer>(p);
    }
    void deallocate(pointer p, size_type) { std::free(p); }
    size_type max_size() const { return size_type(-1) / sizeof(T); }
    template <typename U, typename... A> void construct(U *p, A &&...a) { ::new ((void *)p) U(std::forward<A>(a)...); }
    template <typename U> void destroy(U *p) { p->~U(); }
    bool operator==(const scalable_allocator &) const { return true; }
    bool operator!=(const scalable_allocator &) const { return false; }
};
}  // namespace tbb
