// Learned surrogate of the forward solve: a small 3D convolutional U-Net,
// trained and evaluated with the kernels in this file. Forward and
// data-gradient convolutions run on tcgen05 (k_conv_fwd_tc) by default, or
// on mma.sync tiles (k_conv_fwd); the weight gradient on mma.sync over
// staged tiles (k_conv_wgrad_tiled: its GEMM has M, N = channels <= 64 and
// K = voxels, below tcgen05's smallest M of 64).
//
// Tensors are channels-last, [batch][z][y][x][channel], bf16 activations and
// weights with fp32 accumulation; a layer reads or writes a channel slice
// (offset, stride) of a wider tensor, which is how the U-Net's skip
// concatenations are laid out. Convolutions are 3x3x3, stride 1, zero
// padding, as implicit GEMMs on the tensor cores (mma.sync m16n8k16 bf16):
//   forward      out[v, co]    = sum_{tap, ci} in[v + tap, ci] w[co, tap, ci]
//   data grad    din[v, ci]    = the forward kernel on dout with the weights
//                                flipped in space and transposed in channels
//   weight grad  dw[co, tap, ci] = sum_v dout[v, co] in[v + tap, ci]
//                                (split over voxel chunks, fp32 atomics)
// plus bias/ReLU epilogues, 2x average pooling, 2x nearest upsampling, the
// sigmoid + squared-error loss, and Adam on fp32 master weights.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "gbg_internal.cuh"

namespace gbg {
namespace sg {

struct Geom {
    int B, D, H, W;  // batch and grid
    __host__ __device__ long voxels() const { return (long)B * D * H * W; }
};

struct Slice {
    __nv_bfloat16 *p;  // base of the tensor
    int stride;        // channels per voxel of the tensor
    int off;           // first channel of the slice
};

__device__ __forceinline__ unsigned pack2(__nv_bfloat16 a, __nv_bfloat16 b) {
    return (unsigned)__bfloat16_as_ushort(a) | ((unsigned)__bfloat16_as_ushort(b) << 16);
}

__device__ __forceinline__ void mma16816(float c[4], const unsigned a[4], const unsigned b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// voxel index -> (b, z, y, x)
__device__ __forceinline__ void unflat(const Geom &g, long v, int &b, int &z, int &y, int &x) {
    x = (int)(v % g.W);
    long t = v / g.W;
    y = (int)(t % g.H);
    t /= g.H;
    z = (int)(t % g.D);
    b = (int)(t / g.D);
}

// Forward conv. One warp computes 16 voxels x NT*8 output channels.
// Cin % 16 == 0, Cout == NT*8. w: [Cout][27][Cin] bf16.
template <int NT>
__global__ void __launch_bounds__(128) k_conv_fwd(Geom g, Slice in, int Cin, const __nv_bfloat16 *__restrict__ w,
                                                  const float *__restrict__ bias, Slice out, float *__restrict__ out_f32,
                                                  int relu) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const long v0 = (long)warp * 16;
    const long nv = g.voxels();
    if (v0 >= nv) return;
    const int r0 = lane >> 2, kq = (lane & 3) * 2;
    // the two voxels this thread loads A rows for
    int bb[2], zz[2], yy[2], xx[2];
    bool ok[2];
    for (int h = 0; h < 2; ++h) {
        const long v = v0 + r0 + 8 * h;
        ok[h] = v < nv;
        unflat(g, ok[h] ? v : 0, bb[h], zz[h], yy[h], xx[h]);
    }
    float acc[NT][4];
    for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const int K = 27 * Cin;
    for (int tap = 0; tap < 27; ++tap) {
        const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
        const __nv_bfloat16 *src[2];
        for (int h = 0; h < 2; ++h) {
            const int z = zz[h] + dz, y = yy[h] + dy, x = xx[h] + dx;
            const bool in_b = ok[h] && z >= 0 && z < g.D && y >= 0 && y < g.H && x >= 0 && x < g.W;
            src[h] = in_b ? in.p + ((((long)bb[h] * g.D + z) * g.H + y) * g.W + x) * in.stride + in.off : nullptr;
        }
        for (int c0 = 0; c0 < Cin; c0 += 16) {
            unsigned a[4];
            for (int h = 0; h < 2; ++h) {
                if (src[h]) {
                    a[h] = *reinterpret_cast<const unsigned *>(src[h] + c0 + kq);
                    a[h + 2] = *reinterpret_cast<const unsigned *>(src[h] + c0 + kq + 8);
                } else {
                    a[h] = 0u;
                    a[h + 2] = 0u;
                }
            }
            const int k = tap * Cin + c0;
            for (int j = 0; j < NT; ++j) {
                const __nv_bfloat16 *wr = w + (long)(j * 8 + r0) * K + k + kq;
                unsigned b[2];
                b[0] = *reinterpret_cast<const unsigned *>(wr);
                b[1] = *reinterpret_cast<const unsigned *>(wr + 8);
                mma16816(acc[j], a, b);
            }
        }
    }
    for (int j = 0; j < NT; ++j)
        for (int h = 0; h < 2; ++h) {
            const long v = v0 + r0 + 8 * h;
            if (v >= nv) continue;
            for (int e = 0; e < 2; ++e) {
                const int co = j * 8 + kq + e;
                float val = acc[j][2 * h + e] + (bias ? bias[co] : 0.f);
                if (relu) val = fmaxf(val, 0.f);
                if (out_f32) out_f32[v * (NT * 8) + co] = val;
                if (out.p) out.p[v * out.stride + out.off + co] = __float2bfloat16(val);
            }
        }
}

// ---- forward convolution on the 5th-generation tensor cores (tcgen05) ----------
// Same GEMM as k_conv_fwd: D[v, co] = sum_{tap, ci} in[v + tap, ci] w[co, tap, ci],
// M = 128 voxels per tile, N = Cout, K = 27 Cin in chunks of 16. The weights
// (N x K, bf16) sit in shared memory for the whole launch; the A operand of
// each K-chunk (128 voxels x 16 channels of one tap, zero outside the grid)
// is gathered by the 128 threads into one of S shared-memory stages; one
// thread issues tcgen05.mma (bf16 x bf16 -> fp32 accumulator in tensor
// memory) and commits it to the stage's mbarrier, which frees the stage when
// the MMA has read it. Operands use the no-swizzle K-major layout: 8-row x
// 16-byte core matrices, the two core matrices of a 16-wide K-chunk 128 B
// apart (leading byte offset), 8-row groups 256 B apart (stride byte
// offset). The epilogue reads the accumulator with tcgen05.ld (warp w owns
// tensor-memory lanes 32w..32w+31 = voxels), adds the bias, applies ReLU and
// stores bf16 and/or fp32. Every mbarrier wait is bounded; on a timeout the
// kernel records an error, waits (bounded) for its MMAs and frees its
// tensor memory before leaving.
namespace tc {
constexpr int S = 3;              // A stages
constexpr int G = 3;              // K-chunks per stage (27 Cin / 16 is a multiple of 3)
constexpr int STAGE = G * 4096;   // bytes per stage

__device__ __forceinline__ unsigned saddr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading and stride byte
// offsets (16-byte units), descriptor version 1, no swizzle
__device__ __forceinline__ unsigned long long sdesc(unsigned addr, unsigned lbo, unsigned sbo) {
    return (unsigned long long)((addr >> 4) & 0x3FFFu) | ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
           ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor, kind::f16: fp32 accumulator, bf16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr unsigned idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}

__device__ __forceinline__ void bar_init(unsigned long long *b) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(b)) : "memory");
}
__device__ __forceinline__ bool bar_wait(unsigned long long *b, unsigned parity) {
    for (long long spins = 0; spins < (1ll << 24); ++spins) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(saddr(b)), "r"(parity)
            : "memory");
        if (done) return true;
        if (spins > 64) __nanosleep(32);
    }
    return false;
}
__device__ __forceinline__ void mma(unsigned tmem, unsigned long long a, unsigned long long b, unsigned idesc,
                                    int accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void commit(unsigned long long *b) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(saddr(b))
                 : "memory");
}
__device__ __forceinline__ void ld16(unsigned taddr, unsigned (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

__host__ __device__ constexpr int ncols(int N) { return N < 32 ? 32 : N; }
inline size_t smem_bytes(int Cin, int N) {
    return (size_t)(27 * Cin / 16) * N * 32 + (size_t)S * STAGE + 8 * (S + 1) + 16;
}
}  // namespace tc

template <int N>
__global__ void __launch_bounds__(128) k_conv_fwd_tc(Geom g, Slice in, int Cin, const __nv_bfloat16 *__restrict__ w,
                                                     const float *__restrict__ bias, Slice out,
                                                     float *__restrict__ out_f32, int relu, int *status) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const int K = 27 * Cin, KC = K / 16, CC = Cin / 16;
    unsigned char *Bs = sm;                            // KC chunks of N x 16 bf16
    unsigned char *As = sm + (size_t)KC * N * 32;      // S stages of G x (128 x 16 bf16)
    unsigned long long *bars = reinterpret_cast<unsigned long long *>(As + tc::S * tc::STAGE);  // stages + done
    unsigned *tslot = reinterpret_cast<unsigned *>(bars + tc::S + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    // weights into the core-matrix layout, 16-byte pieces (8 consecutive k of one n)
    for (int pc = tid; pc < N * (K / 8); pc += 128) {
        const int n = pc / (K / 8), k8 = pc % (K / 8);
        unsigned char *dst = Bs + (size_t)(k8 >> 1) * N * 32 + (n >> 3) * 256 + (k8 & 1) * 128 + (n & 7) * 16;
        *reinterpret_cast<uint4 *>(dst) = *reinterpret_cast<const uint4 *>(w + (size_t)n * K + (size_t)k8 * 8);
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    if (tid == 0) {
        for (int i = 0; i <= tc::S; ++i) tc::bar_init(bars + i);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tc::saddr(tslot)),
                     "r"(tc::ncols(N))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const unsigned tmem = *tslot;
    constexpr unsigned IDESC = tc::idesc_bf16(128, N);
    const long nv = g.voxels();
    const long tiles = (nv + 127) / 128;
    long gc = 0;             // K-chunks issued by this CTA (stage = gc % S)
    unsigned done_phase = 0;
    bool ok = true;
    for (long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const long v = tile * 128 + tid;
        const bool valid = v < nv;
        int bb = 0, z = 0, y = 0, x = 0;
        unflat(g, valid ? v : 0, bb, z, y, x);
        // K-chunks in groups of G per stage; the next group's global loads are
        // issued before the barrier that hands the current group to the MMA
        uint4 pre[2 * tc::G];
        auto load_group = [&](int gi) {
#pragma unroll
            for (int j = 0; j < tc::G; ++j) {
                const int c = gi * tc::G + j;
                const int tap = c / CC, ci0 = (c % CC) * 16;
                const int zz = z + tap / 9 - 1, yy = y + (tap / 3) % 3 - 1, xx = x + tap % 3 - 1;
                uint4 lo = make_uint4(0, 0, 0, 0), hi = lo;
                if (valid && zz >= 0 && zz < g.D && yy >= 0 && yy < g.H && xx >= 0 && xx < g.W) {
                    const __nv_bfloat16 *src =
                        in.p + ((((long)bb * g.D + zz) * g.H + yy) * g.W + xx) * in.stride + in.off + ci0;
                    lo = *reinterpret_cast<const uint4 *>(src);
                    hi = *reinterpret_cast<const uint4 *>(src + 8);
                }
                pre[2 * j] = lo;
                pre[2 * j + 1] = hi;
            }
        };
        const int NGRP = KC / tc::G;
        load_group(0);
        for (int gi = 0; gi < NGRP; ++gi, ++gc) {
            const int s = (int)(gc % tc::S);
            bool okw = true;
            if (gc >= tc::S) okw = tc::bar_wait(bars + s, (unsigned)((gc / tc::S - 1) & 1));
            unsigned char *stage = As + (size_t)s * tc::STAGE;
#pragma unroll
            for (int j = 0; j < tc::G; ++j) {
                unsigned char *a = stage + j * 4096 + (tid >> 3) * 256 + (tid & 7) * 16;
                *reinterpret_cast<uint4 *>(a) = pre[2 * j];
                *reinterpret_cast<uint4 *>(a + 128) = pre[2 * j + 1];
            }
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            if (gi + 1 < NGRP) load_group(gi + 1);
            if (__syncthreads_or(!okw)) {
                ok = false;
                break;
            }
            if (tid == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
                for (int j = 0; j < tc::G; ++j) {
                    const int c = gi * tc::G + j;
                    const unsigned long long ad = tc::sdesc(tc::saddr(stage + j * 4096), 128, 256);
                    const unsigned long long bd = tc::sdesc(tc::saddr(Bs + (size_t)c * N * 32), 128, 256);
                    tc::mma(tmem, ad, bd, IDESC, c > 0 ? 1 : 0);
                }
                tc::commit(bars + s);
            }
        }
        if (!ok) break;
        if (tid == 0) tc::commit(bars + tc::S);
        const bool okd = tc::bar_wait(bars + tc::S, done_phase);
        done_phase ^= 1u;
        if (__syncthreads_or(!okd)) {
            ok = false;
            break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        unsigned r[N];
#pragma unroll
        for (int q = 0; q < N / 16; ++q) {
            unsigned part[16];
            tc::ld16(tmem + ((unsigned)(32 * warp) << 16) + 16 * q, part);
#pragma unroll
            for (int e = 0; e < 16; ++e) r[16 * q + e] = part[e];
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        if (valid) {
#pragma unroll
            for (int co = 0; co < N; ++co) {
                float val = __uint_as_float(r[co]) + (bias ? bias[co] : 0.f);
                if (relu) val = fmaxf(val, 0.f);
                if (out_f32) out_f32[v * N + co] = val;
                if (out.p) out.p[v * out.stride + out.off + co] = __float2bfloat16(val);
            }
        }
        // every warp has read the accumulator before the next tile's first MMA
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
    }
    if (!ok) {
        if (tid == 0) {
            atomicExch(status, (int)DEV_MMA_TIMEOUT);
            tc::commit(bars + tc::S);
        }
        tc::bar_wait(bars + tc::S, done_phase);  // the MMAs issued so far (bounded)
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(tc::ncols(N))
                     : "memory");
}

// Halo-tile variant (grids with W % 8 == 0 and H % 16 == 0): an output tile
// is 8 (x) x 16 (y) voxels of one z-plane of one sample, M = 128 rows ordered
// x-fastest. Its input halo, 10 (x) x 18 (y) x 3 (z) voxels, is loaded into
// shared memory once, one array per 8-channel chunk, voxels x-fastest at 16
// bytes each: 8 consecutive x-voxels of a chunk are one 128-byte core matrix.
// The A operand of tap (dx, dy, dz) is then a descriptor into the halo tile
// (start = the tap's offset, stride byte offset = one halo row = 160 B,
// leading byte offset = one chunk array), so all 27 Cin / 16 MMAs of a tile
// are issued back to back without gathering.
namespace tc {
constexpr int HX = 10, HY = 18, HZ = 3;
constexpr int HALO_CHUNK = HX * HY * HZ * 16;  // bytes per 8-channel chunk array (8640)
inline size_t halo_smem_bytes(int Cin, int N) {  // weights, two halo buffers, barrier, tmem slot
    return (size_t)(27 * Cin / 16) * N * 32 + 2 * (size_t)(Cin / 8) * HALO_CHUNK + 8 * 2 + 16;
}
}  // namespace tc

template <int N>
__global__ void __launch_bounds__(128) k_conv_fwd_tc_halo(Geom g, Slice in, int Cin, const __nv_bfloat16 *__restrict__ w,
                                                          const float *__restrict__ bias, Slice out,
                                                          float *__restrict__ out_f32, int relu, int *status) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const int K = 27 * Cin, KC = K / 16, CC = Cin / 16, C8 = Cin / 8;
    unsigned char *Bs = sm;                                   // KC chunks of N x 16 bf16
    unsigned char *Hs = sm + (size_t)KC * N * 32;             // two halo tiles of C8 chunk arrays
    unsigned long long *bars = reinterpret_cast<unsigned long long *>(Hs + 2 * (size_t)C8 * tc::HALO_CHUNK);
    unsigned *tslot = reinterpret_cast<unsigned *>(bars + 2);
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int pc = tid; pc < N * (K / 8); pc += 128) {
        const int n = pc / (K / 8), k8 = pc % (K / 8);
        unsigned char *dst = Bs + (size_t)(k8 >> 1) * N * 32 + (n >> 3) * 256 + (k8 & 1) * 128 + (n & 7) * 16;
        *reinterpret_cast<uint4 *>(dst) = *reinterpret_cast<const uint4 *>(w + (size_t)n * K + (size_t)k8 * 8);
    }
    if (tid == 0) {
        tc::bar_init(bars);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tc::saddr(tslot)),
                     "r"(tc::ncols(N))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const unsigned tmem = *tslot;
    constexpr unsigned IDESC = tc::idesc_bf16(128, N);
    const int tx = g.W / 8, ty = g.H / 16;
    const long tiles = (long)g.B * g.D * ty * tx;
    const size_t halo_bytes = (size_t)C8 * tc::HALO_CHUNK;
    // halo tile of `tile` into buffer `buf` (each thread fences its own stores)
    auto load_tile = [&](long tile, int buf) {
        const int x0 = (int)(tile % tx) * 8;
        long t = tile / tx;
        const int y0 = (int)(t % ty) * 16;
        t /= ty;
        const int z = (int)(t % g.D);
        const int bb = (int)(t / g.D);
        unsigned char *H = Hs + (size_t)buf * halo_bytes;
        const int entries = C8 * tc::HX * tc::HY * tc::HZ;
        for (int e = tid; e < entries; e += 128) {
            const int hx = e % tc::HX;
            int r = e / tc::HX;
            const int hy = r % tc::HY;
            r /= tc::HY;
            const int hz = r % tc::HZ, k8 = r / tc::HZ;
            const int xx = x0 + hx - 1, yy = y0 + hy - 1, zz = z + hz - 1;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (xx >= 0 && xx < g.W && yy >= 0 && yy < g.H && zz >= 0 && zz < g.D)
                v = *reinterpret_cast<const uint4 *>(
                    in.p + ((((long)bb * g.D + zz) * g.H + yy) * g.W + xx) * in.stride + in.off + k8 * 8);
            *reinterpret_cast<uint4 *>(H + (size_t)k8 * tc::HALO_CHUNK + ((hz * tc::HY + hy) * tc::HX + hx) * 16) = v;
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    };
    unsigned done_phase = 0;
    bool ok = true;
    int buf = 0;
    if (blockIdx.x < tiles) load_tile(blockIdx.x, 0);
    __syncthreads();
    for (long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x, buf ^= 1) {
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const unsigned char *H = Hs + (size_t)buf * halo_bytes;
            for (int tap = 0; tap < 27; ++tap) {
                const int dx = tap % 3, dy = (tap / 3) % 3, dz = tap / 9;  // halo offsets of the tap
                const unsigned toff = ((dz * tc::HY + dy) * tc::HX + dx) * 16;
                for (int cc = 0; cc < CC; ++cc) {
                    const int c = tap * CC + cc;
                    // K-chunk cc = channel chunks 2cc and 2cc+1: leading byte offset = one chunk array
                    const unsigned long long ad =
                        tc::sdesc(tc::saddr(H + (size_t)(2 * cc) * tc::HALO_CHUNK + toff), tc::HALO_CHUNK, tc::HX * 16);
                    const unsigned long long bd = tc::sdesc(tc::saddr(Bs + (size_t)c * N * 32), 128, 256);
                    tc::mma(tmem, ad, bd, IDESC, c > 0 ? 1 : 0);
                }
            }
            tc::commit(bars);
        }
        // the next tile's halo goes to the other buffer while the MMAs run
        // (that buffer's previous MMAs completed before the last epilogue)
        if (tile + gridDim.x < tiles) load_tile(tile + gridDim.x, buf ^ 1);
        const bool okd = tc::bar_wait(bars, done_phase);
        done_phase ^= 1u;
        if (__syncthreads_or(!okd)) {
            ok = false;
            break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        unsigned r[N];
#pragma unroll
        for (int q = 0; q < N / 16; ++q) {
            unsigned part[16];
            tc::ld16(tmem + ((unsigned)(32 * warp) << 16) + 16 * q, part);
#pragma unroll
            for (int e = 0; e < 16; ++e) r[16 * q + e] = part[e];
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        // row m = tid: x = x0 + m % 8, y = y0 + m / 8
        {
            const int x0 = (int)(tile % tx) * 8;
            long t = tile / tx;
            const int y0 = (int)(t % ty) * 16;
            t /= ty;
            const int z = (int)(t % g.D);
            const int bb = (int)(t / g.D);
            const long v = (((long)bb * g.D + z) * g.H + (y0 + tid / 8)) * g.W + (x0 + tid % 8);
            float val[N];
#pragma unroll
            for (int co = 0; co < N; ++co) {
                val[co] = __uint_as_float(r[co]) + (bias ? bias[co] : 0.f);
                if (relu) val[co] = fmaxf(val[co], 0.f);
            }
            if (out_f32) {
#pragma unroll
                for (int q = 0; q < N / 4; ++q)
                    *reinterpret_cast<float4 *>(out_f32 + v * N + 4 * q) =
                        make_float4(val[4 * q], val[4 * q + 1], val[4 * q + 2], val[4 * q + 3]);
            }
            if (out.p) {
                // 8 channels per 16-byte store (the slice offset and stride are multiples of 8)
#pragma unroll
                for (int q = 0; q < N / 8; ++q) {
                    uint4 pk;
                    pk.x = pack2(__float2bfloat16(val[8 * q]), __float2bfloat16(val[8 * q + 1]));
                    pk.y = pack2(__float2bfloat16(val[8 * q + 2]), __float2bfloat16(val[8 * q + 3]));
                    pk.z = pack2(__float2bfloat16(val[8 * q + 4]), __float2bfloat16(val[8 * q + 5]));
                    pk.w = pack2(__float2bfloat16(val[8 * q + 6]), __float2bfloat16(val[8 * q + 7]));
                    *reinterpret_cast<uint4 *>(out.p + v * out.stride + out.off + 8 * q) = pk;
                }
            }
        }
        // the accumulator is read, and the next halo stored, before the next tile's MMAs
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
    }
    if (!ok) {
        if (tid == 0) atomicExch(status, (int)DEV_MMA_TIMEOUT);
        tc::bar_wait(bars, done_phase);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(tc::ncols(N))
                     : "memory");
}

// Weight gradient for one tap: dw[co][tap][ci] += sum_v dout[v][co] * in[v+tap][ci].
// M = Cout (16-row tiles), N = Cin (8-col tiles), K = voxels in chunks of 16.
// Each warp handles one (m-tile, n-tile) over a voxel range.
__global__ void __launch_bounds__(128) k_conv_wgrad(Geom g, Slice in, int Cin, Slice dout, int Cout, long chunk,
                                                    float *__restrict__ dw) {
    const int lane = threadIdx.x & 31;
    const int warp_in_cta = threadIdx.x >> 5;
    const int mt_n = Cout / 16, nt_n = Cin / 8;
    const int tiles = 27 * mt_n * nt_n;
    const int tile = blockIdx.y * 4 + warp_in_cta;
    if (tile >= tiles) return;
    const int tap = tile / (mt_n * nt_n);
    const int mt = (tile / nt_n) % mt_n, nt = tile % nt_n;
    const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
    const long nv = g.voxels();
    const long vbeg = (long)blockIdx.x * chunk, vend = vbeg + chunk < nv ? vbeg + chunk : nv;
    const int r0 = lane >> 2, kq = (lane & 3) * 2;
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    for (long vk = vbeg; vk < vend; vk += 16) {
        // A: rows co = mt*16 + r0 (+8), cols voxel vk + kq (+1, +8, +9)
        // B: rows voxel vk + kq (+1, +8, +9), col ci = nt*8 + r0
        __nv_bfloat16 av[2][4], bv[4];
        for (int q = 0; q < 4; ++q) {
            const long v = vk + kq + (q & 1) + (q >> 1) * 8;
            __nv_bfloat16 a0 = __float2bfloat16(0.f), a1 = a0, bvq = a0;
            if (v < vend) {
                a0 = dout.p[v * dout.stride + dout.off + mt * 16 + r0];
                a1 = dout.p[v * dout.stride + dout.off + mt * 16 + r0 + 8];
                int b, z, y, x;
                unflat(g, v, b, z, y, x);
                z += dz; y += dy; x += dx;
                if (z >= 0 && z < g.D && y >= 0 && y < g.H && x >= 0 && x < g.W)
                    bvq = in.p[((((long)b * g.D + z) * g.H + y) * g.W + x) * in.stride + in.off + nt * 8 + r0];
            }
            av[0][q] = a0;
            av[1][q] = a1;
            bv[q] = bvq;
        }
        unsigned a[4], bf[2];
        a[0] = pack2(av[0][0], av[0][1]);
        a[1] = pack2(av[1][0], av[1][1]);
        a[2] = pack2(av[0][2], av[0][3]);
        a[3] = pack2(av[1][2], av[1][3]);
        bf[0] = pack2(bv[0], bv[1]);
        bf[1] = pack2(bv[2], bv[3]);
        mma16816(c, a, bf);
    }
    // c[0..1]: row co = mt*16 + r0, cols ci = nt*8 + kq + {0,1}; c[2..3]: row + 8
    const int K = 27 * Cin;
    for (int h = 0; h < 2; ++h)
        for (int e = 0; e < 2; ++e) {
            const int co = mt * 16 + r0 + 8 * h, ci = nt * 8 + kq + e;
            atomicAdd(dw + (long)co * K + tap * Cin + ci, c[2 * h + e]);
        }
}

// Weight gradient on staged tiles. A persistent CTA (8 warps) walks voxel
// tiles of 8 (x) x 8 (y) of one z-plane; per tile it stages the input's
// 10 x 10 x 3 halo and the tile's output gradient in shared memory (16-byte
// loads, rows padded by 8 channels so that ldmatrix rows fall in distinct
// banks) and accumulates, for every (tap, 16 output channels, 8 input
// channels) block it owns, dw += dout^T(16 x 16 voxels) in_tap(16 voxels x 8)
// with mma.sync m16n8k16. Fragments come from ldmatrix.trans (both operands
// are stored voxel-major, channels contiguous); the tap's shift is the row
// addresses of the B fragment. Accumulators stay in registers over all of a
// CTA's tiles and are added to dw (fp32 atomics) once at the end.
// Needs W % 8 == 0, H % 8 == 0, slice strides and offsets multiples of 8.
__device__ __forceinline__ void ldsm_x4_trans(unsigned r[4], const void *p) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

__device__ __forceinline__ void ldsm_x2_trans(unsigned r[2], const void *p) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
                 : "=r"(r[0]), "=r"(r[1])
                 : "r"(a));
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_conv_wgrad_tiled(Geom g, Slice in, Slice dout, float *__restrict__ dw) {
    constexpr int TX = 8, TY = 8, TV = TX * TY;
    constexpr int HX = TX + 2, HY = TY + 2, HV = 3 * HY * HX;
    constexpr int CP = CIN + 8, OP = COUT + 8;  // padded voxel strides (elements)
    // a warp owns the (tap, 8 input channels) blocks warp, warp + 8, ... for
    // every group of 16 output channels (the B fragment serves them all)
    constexpr int CT = COUT / 16, NT = CIN / 8, TN = 27 * NT, NW = 8;
    constexpr int TPW = (TN + NW - 1) / NW;
    __shared__ __align__(16) __nv_bfloat16 sh_in[HV * CP];
    __shared__ __align__(16) __nv_bfloat16 sh_out[TV * OP];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int q = lane >> 3, i8 = lane & 7;
    float acc[CT][TPW][4];
#pragma unroll
    for (int ct = 0; ct < CT; ++ct)
#pragma unroll
        for (int j = 0; j < TPW; ++j) acc[ct][j][0] = acc[ct][j][1] = acc[ct][j][2] = acc[ct][j][3] = 0.f;
    const int tx_n = g.W / TX, ty_n = g.H / TY;
    const long ntiles = (long)g.B * g.D * ty_n * tx_n;
    for (long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int xt = (int)(t % tx_n);
        long r = t / tx_n;
        const int yt = (int)(r % ty_n);
        r /= ty_n;
        const int z = (int)(r % g.D), b = (int)(r / g.D);
        const int x0 = xt * TX, y0 = yt * TY;
        __syncthreads();  // the previous tile's fragments are read
        for (int k = threadIdx.x; k < HV * (CIN / 8); k += blockDim.x) {
            const int c8 = k % (CIN / 8), hv = k / (CIN / 8);
            const int hx = hv % HX, hy = (hv / HX) % HY, hz = hv / (HX * HY);
            const int X = x0 + hx - 1, Y = y0 + hy - 1, Z = z + hz - 1;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (X >= 0 && X < g.W && Y >= 0 && Y < g.H && Z >= 0 && Z < g.D)
                v = *reinterpret_cast<const uint4 *>(in.p + ((((long)b * g.D + Z) * g.H + Y) * g.W + X) * in.stride +
                                                     in.off + c8 * 8);
            *reinterpret_cast<uint4 *>(sh_in + hv * CP + c8 * 8) = v;
        }
        for (int k = threadIdx.x; k < TV * (COUT / 8); k += blockDim.x) {
            const int c8 = k % (COUT / 8), vv = k / (COUT / 8);
            const int X = x0 + vv % TX, Y = y0 + vv / TX;
            *reinterpret_cast<uint4 *>(sh_out + vv * OP + c8 * 8) = *reinterpret_cast<const uint4 *>(
                dout.p + ((((long)b * g.D + z) * g.H + Y) * g.W + X) * dout.stride + dout.off + c8 * 8);
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < TV / 16; ++ks) {
            // A = dout^T for 16 voxels (rows 2ks, 2ks+1 of the tile): matrix q
            // covers channels (q & 1) * 8 .. +7 and voxels (q >> 1) * 8 .. +7
            unsigned a[CT][4];
#pragma unroll
            for (int ct = 0; ct < CT; ++ct)
                ldsm_x4_trans(a[ct], sh_out + (ks * 16 + (q >> 1) * 8 + i8) * OP + ct * 16 + (q & 1) * 8);
            // B rows: voxel (x = i8, y = 2ks + (q & 1)) shifted by the tap
            const int vy = 2 * ks + (q & 1);
#pragma unroll
            for (int j = 0; j < TPW; ++j) {
                const int tl = warp + j * NW;
                if (tl < TN) {
                    const int tap = tl / NT, nt = tl % NT;
                    const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
                    const int hidx = ((dz + 1) * HY + (vy + dy + 1)) * HX + (i8 + dx + 1);
                    unsigned bf[2];
                    ldsm_x2_trans(bf, sh_in + hidx * CP + nt * 8);
#pragma unroll
                    for (int ct = 0; ct < CT; ++ct) mma16816(acc[ct][j], a[ct], bf);
                }
            }
        }
    }
    const int K = 27 * CIN, r0 = lane >> 2, kq = (lane & 3) * 2;
#pragma unroll
    for (int j = 0; j < TPW; ++j) {
        const int tl = warp + j * NW;
        if (tl < TN) {
            const int tap = tl / NT, nt = tl % NT;
#pragma unroll
            for (int ct = 0; ct < CT; ++ct)
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int e = 0; e < 2; ++e) {
                        const int co = ct * 16 + r0 + 8 * h, ci = nt * 8 + kq + e;
                        atomicAdd(dw + (long)co * K + tap * CIN + ci, acc[ct][j][2 * h + e]);
                    }
        }
    }
}

// flipped/transposed weights for the data gradient: wt[ci][26-tap][co] = w[co][tap][ci]
__global__ void k_flip_weights(const __nv_bfloat16 *__restrict__ w, int Cout, int Cin, __nv_bfloat16 *__restrict__ wt) {
    const long n = (long)Cout * 27 * Cin;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int ci = (int)(i % Cin), tap = (int)((i / Cin) % 27), co = (int)(i / (27L * Cin));
        wt[((long)ci * 27 + (26 - tap)) * Cout + co] = w[i];
    }
}

// dY *= (Y > 0) on a slice (ReLU backward, Y the layer's output)
__global__ void k_relu_bwd(long nv, int C, Slice y, Slice dy) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nv * C; i += (long)gridDim.x * blockDim.x) {
        const long v = i / C;
        const int c = (int)(i % C);
        if (!(__bfloat162float(y.p[v * y.stride + y.off + c]) > 0.f)) dy.p[v * dy.stride + dy.off + c] = __float2bfloat16(0.f);
    }
}

__global__ void k_bias_grad(long nv, int C, Slice dy, float *__restrict__ db) {
    __shared__ float red[256];
    const int c = blockIdx.y;
    float s = 0.f;
    for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < nv; v += (long)gridDim.x * blockDim.x)
        s += __bfloat162float(dy.p[v * dy.stride + dy.off + c]);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(db + c, red[0]);
}

// 2x average pooling: out (D/2, H/2, W/2) <- in; and its transpose
__global__ void k_pool2(Geom go, int C, Slice in, Slice out) {
    const long n = go.voxels() * C;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const long v = i / C;
        const int c = (int)(i % C);
        int b, z, y, x;
        unflat(go, v, b, z, y, x);
        const int Hi = go.H * 2, Wi = go.W * 2, Di = go.D * 2;
        float s = 0.f;
        for (int q = 0; q < 8; ++q) {
            const long vi = (((long)b * Di + 2 * z + (q >> 2)) * Hi + 2 * y + ((q >> 1) & 1)) * Wi + 2 * x + (q & 1);
            s += __bfloat162float(in.p[vi * in.stride + in.off + c]);
        }
        out.p[v * out.stride + out.off + c] = __float2bfloat16(0.125f * s);
    }
}

__global__ void k_pool2_bwd(Geom gi, int C, Slice dout, Slice din) {
    const long n = gi.voxels() * C;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const long v = i / C;
        const int c = (int)(i % C);
        int b, z, y, x;
        unflat(gi, v, b, z, y, x);
        const long vo = (((long)b * (gi.D / 2) + z / 2) * (gi.H / 2) + y / 2) * (gi.W / 2) + x / 2;
        din.p[v * din.stride + din.off + c] = __float2bfloat16(0.125f * __bfloat162float(dout.p[vo * dout.stride + dout.off + c]));
    }
}

// 2x nearest upsampling: out (fine) <- in (coarse); and its transpose (sum of 8)
__global__ void k_up2(Geom gf, int C, Slice in, Slice out) {
    // 8 channels (16 bytes) per item: C, the strides and offsets are multiples of 8
    const int C8 = C / 8;
    const long n = gf.voxels() * C8;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const long v = i / C8;
        const int c = (int)(i % C8) * 8;
        int b, z, y, x;
        unflat(gf, v, b, z, y, x);
        const long vc = (((long)b * (gf.D / 2) + z / 2) * (gf.H / 2) + y / 2) * (gf.W / 2) + x / 2;
        *reinterpret_cast<uint4 *>(out.p + v * out.stride + out.off + c) =
            *reinterpret_cast<const uint4 *>(in.p + vc * in.stride + in.off + c);
    }
}

__global__ void k_up2_bwd(Geom gc, int C, Slice dout, Slice din) {
    const long n = gc.voxels() * C;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const long v = i / C;
        const int c = (int)(i % C);
        int b, z, y, x;
        unflat(gc, v, b, z, y, x);
        const int Hf = gc.H * 2, Wf = gc.W * 2, Df = gc.D * 2;
        float s = 0.f;
        for (int q = 0; q < 8; ++q) {
            const long vf = (((long)b * Df + 2 * z + (q >> 2)) * Hf + 2 * y + ((q >> 1) & 1)) * Wf + 2 * x + (q & 1);
            s += __bfloat162float(dout.p[vf * dout.stride + dout.off + c]);
        }
        din.p[v * din.stride + din.off + c] = __float2bfloat16(s);
    }
}

// sigmoid output and squared-error loss against targets: loss += sum (s - t)^2 / nv,
// dlogit = 2 (s - t) s (1 - s) / nv (scaled by loss_scale for bf16 range)
// pred may be logit itself (in-place sigmoid): neither is declared restrict
__global__ void k_loss(long nv, const float *logit, const float *__restrict__ target, float *pred,
                       __nv_bfloat16 *__restrict__ dlogit, float loss_scale, double *__restrict__ loss) {
    __shared__ double red[256];
    double s_acc = 0.0;
    for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < nv; v += (long)gridDim.x * blockDim.x) {
        const float s = 1.f / (1.f + expf(-logit[v]));
        if (pred) pred[v] = s;
        if (target) {
            const float d = s - target[v];
            s_acc += (double)d * d;
            if (dlogit) dlogit[v] = __float2bfloat16(loss_scale * 2.f * d * s * (1.f - s) / (float)nv);
        }
    }
    red[threadIdx.x] = s_acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0 && loss) atomicAdd(loss, red[0] / (double)nv);
}

__global__ void k_adam(long n, float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, __nv_bfloat16 *__restrict__ wb, float lr, float b1, float b2, float eps,
                       float c1, float c2, float gscale) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float gi = g[i] * gscale;
        m[i] = b1 * m[i] + (1.f - b1) * gi;
        v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
        w[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
        if (wb) wb[i] = __float2bfloat16(w[i]);
    }
}

__global__ void k_f32_to_bf16(long n, const float *__restrict__ a, __nv_bfloat16 *__restrict__ b) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        b[i] = __float2bfloat16(a[i]);
}

// Input features at the surrogate grid (n^3, channels padded to 16):
//  0 p_w, 1 p_g, 2 seed blob exp(-|x-x0|^2/(2 s^2)), 3 Dw, 4 rho, 5 T (scaled
//  to [0,1] by the prior ranges), 6 (distance to seed - Fisher-KPP front
//  radius 2 sqrt(Dw rho) T) / 16 voxels, 7..15 zero. Positions, Dw and the
//  radius are in the solver's voxel units; the surrogate grid is `factor`
//  times coarser.
struct FeatParams {
    double dw_lo, dw_hi, rho_lo, rho_hi, t_lo, t_hi, L, n_solver, blob_sigma;
};

__global__ void k_features(int S, int n, int factor, const gbg_sample *__restrict__ smp,
                           const float *__restrict__ pw, const float *__restrict__ pg, FeatParams fp,
                           __nv_bfloat16 *__restrict__ x) {
    const long N = (long)n * n * n;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N * S; i += (long)gridDim.x * blockDim.x) {
        const long s = i / N, c = i % N;
        const int xx = (int)(c % n), yy = (int)((c / n) % n), zz = (int)(c / ((long)n * n));
        const gbg_sample q = smp[s];
        // per-sample scalars in double; per-cell geometry in float (the
        // features are rounded to bf16)
        // front speed 2 sqrt(D rho) in voxels/day: D in voxel^2/day = Dw / L^2 * n_solver^2
        const double dvox = q.Dw / (fp.L * fp.L) * fp.n_solver * fp.n_solver;
        const float front = (float)(2.0 * sqrt(dvox * q.rho) * q.tend);
        const float inv2s2 = (float)(1.0 / (2.0 * fp.blob_sigma * fp.blob_sigma));
        // cell centre in solver voxel units
        const float dx = (float)((xx + 0.5) * factor - 0.5 - q.x0), dy = (float)((yy + 0.5) * factor - 0.5 - q.y0),
                    dz = (float)((zz + 0.5) * factor - 0.5 - q.z0);
        const float d2 = dx * dx + dy * dy + dz * dz;
        const float f[7] = {pw[c], pg[c], expf(-d2 * inv2s2), (float)((q.Dw - fp.dw_lo) / (fp.dw_hi - fp.dw_lo)),
                            (float)((q.rho - fp.rho_lo) / (fp.rho_hi - fp.rho_lo)),
                            (float)((q.tend - fp.t_lo) / (fp.t_hi - fp.t_lo)), (sqrtf(d2) - front) * (1.0f / 16.0f)};
        uint4 lo, hi = make_uint4(0, 0, 0, 0);
        lo.x = pack2(__float2bfloat16(f[0]), __float2bfloat16(f[1]));
        lo.y = pack2(__float2bfloat16(f[2]), __float2bfloat16(f[3]));
        lo.z = pack2(__float2bfloat16(f[4]), __float2bfloat16(f[5]));
        lo.w = pack2(__float2bfloat16(f[6]), __float2bfloat16(0.f));
        uint4 *o = reinterpret_cast<uint4 *>(x + i * 16);
        o[0] = lo;
        o[1] = hi;
    }
}

// 2x average pooling of S float fields n^3 -> (n/2)^3
__global__ void k_down2_f32(int S, int n, const float *__restrict__ in, float *__restrict__ out) {
    const int m = n / 2;
    const long M = (long)m * m * m;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < M * S; i += (long)gridDim.x * blockDim.x) {
        const long s = i / M, c = i % M;
        const int x = (int)(c % m), y = (int)((c / m) % m), z = (int)(c / ((long)m * m));
        float acc = 0.f;
        for (int q = 0; q < 8; ++q)
            acc += in[s * (long)n * n * n + ((long)(2 * z + (q >> 2)) * n + 2 * y + ((q >> 1) & 1)) * n + 2 * x + (q & 1)];
        out[i] = 0.125f * acc;
    }
}

// nearest 2x upsampling of S float fields m^3 -> (2m)^3, zero outside tissue
__global__ void k_up2_f32(int S, int m, const float *__restrict__ in, const float *__restrict__ mask,
                          float *__restrict__ out) {
    const int n = 2 * m;
    const long N = (long)n * n * n;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N * S; i += (long)gridDim.x * blockDim.x) {
        const long s = i / N, c = i % N;
        const int x = (int)(c % n), y = (int)((c / n) % n), z = (int)(c / ((long)n * n));
        const float v = in[s * (long)m * m * m + ((long)(z / 2) * m + y / 2) * m + x / 2];
        out[i] = mask[c] != 0.f ? v : 0.f;
    }
}

}  // namespace sg
}  // namespace gbg

// ------------------------------------------------------------------------------
// The network and its training loop.
//
// Surrogate grid m^3 with m = n_solver / factor. Layers (channels):
//   e0a  conv 16->16 relu   x0            -> t0
//   e0b  conv 16->16 relu   t0            -> c0[16:32]
//   pool                    c0[16:32]     -> p1        (m/2)^3
//   e1a  conv 16->32 relu   p1            -> t1
//   e1b  conv 32->32 relu   t1            -> c1[32:64]
//   pool                    c1[32:64]     -> p2        (m/4)^3
//   mid  conv 32->32 relu   p2            -> q2
//   up                      q2            -> c1[0:32]
//   d1   conv 64->16 relu   c1            -> u1
//   up                      u1            -> c0[0:16]
//   d0   conv 32->16 relu   c0            -> u0
//   out  conv 16->16        u0            -> logits (fp32, channel 0 used)
// prediction = sigmoid(logit 0), loss = mean squared error against the
// solver's final density averaged onto the surrogate grid.
namespace gbg {
namespace sg {

struct Layer {
    int cin, cout;
    bool relu;
    long w_off, b_off;  // offsets into the flat parameter vector
};

struct Net {
    std::vector<Layer> L;
    long nparams = 0;
    void add(int ci, int co, bool relu) {
        Layer l{ci, co, relu, nparams, 0};
        nparams += (long)co * 27 * ci;
        l.b_off = nparams;
        nparams += co;
        L.push_back(l);
    }
    Net() {
        add(16, 16, true);   // 0 e0a
        add(16, 16, true);   // 1 e0b
        add(16, 32, true);   // 2 e1a
        add(32, 32, true);   // 3 e1b
        add(32, 32, true);   // 4 mid
        add(64, 16, true);   // 5 d1
        add(32, 16, true);   // 6 d0
        add(16, 16, false);  // 7 out
    }
};

inline int grid_n(long work, int cap = 4096) {
    long g = (work + 255) / 256;
    return (int)(g < cap ? g : cap);
}

// engine 1: tcgen05 kernel (Cout 16, 32 or 64); engine 0: mma.sync kernel
void conv_fwd(cudaStream_t st, Geom g, Slice in, int cin, const __nv_bfloat16 *w, const float *b, Slice out,
              float *out32, int cout, bool relu, int engine = 0, int num_sms = 0, int *status = nullptr) {
    if (engine == 1 && (cout == 16 || cout == 32 || cout == 64) && status && g.W % 8 == 0 && g.H % 16 == 0) {
        const size_t sm = tc::halo_smem_bytes(cin, cout);
        const long tiles = (long)g.B * g.D * (g.H / 16) * (g.W / 8);
        const int grid = (int)std::min<long>(tiles, (long)num_sms * 8);
        const void *fn = cout == 16 ? (const void *)k_conv_fwd_tc_halo<16>
                                    : (cout == 32 ? (const void *)k_conv_fwd_tc_halo<32>
                                                  : (const void *)k_conv_fwd_tc_halo<64>);
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        switch (cout) {
            case 16: k_conv_fwd_tc_halo<16><<<grid, 128, sm, st>>>(g, in, cin, w, b, out, out32, relu, status); break;
            case 32: k_conv_fwd_tc_halo<32><<<grid, 128, sm, st>>>(g, in, cin, w, b, out, out32, relu, status); break;
            case 64: k_conv_fwd_tc_halo<64><<<grid, 128, sm, st>>>(g, in, cin, w, b, out, out32, relu, status); break;
        }
        return;
    }
    if (engine == 1 && (cout == 16 || cout == 32 || cout == 64) && status) {
        const size_t sm = tc::smem_bytes(cin, cout);
        const long tiles = (g.voxels() + 127) / 128;
        const int grid = (int)std::min<long>(tiles, (long)num_sms * 8);
        const void *fn = cout == 16 ? (const void *)k_conv_fwd_tc<16>
                                    : (cout == 32 ? (const void *)k_conv_fwd_tc<32> : (const void *)k_conv_fwd_tc<64>);
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        switch (cout) {
            case 16: k_conv_fwd_tc<16><<<grid, 128, sm, st>>>(g, in, cin, w, b, out, out32, relu, status); break;
            case 32: k_conv_fwd_tc<32><<<grid, 128, sm, st>>>(g, in, cin, w, b, out, out32, relu, status); break;
            case 64: k_conv_fwd_tc<64><<<grid, 128, sm, st>>>(g, in, cin, w, b, out, out32, relu, status); break;
        }
        return;
    }
    const long warps = (g.voxels() + 15) / 16;
    const int ctas = (int)((warps + 3) / 4);
    switch (cout / 8) {
        case 1: k_conv_fwd<1><<<ctas, 128, 0, st>>>(g, in, cin, w, b, out, out32, relu); break;
        case 2: k_conv_fwd<2><<<ctas, 128, 0, st>>>(g, in, cin, w, b, out, out32, relu); break;
        case 4: k_conv_fwd<4><<<ctas, 128, 0, st>>>(g, in, cin, w, b, out, out32, relu); break;
        case 8: k_conv_fwd<8><<<ctas, 128, 0, st>>>(g, in, cin, w, b, out, out32, relu); break;
    }
}

template <int CIN, int COUT>
void wgrad_tiled(cudaStream_t st, Geom g, Slice in, Slice dout, float *dw, int num_sms) {
    const long ntiles = (long)g.B * g.D * (g.H / 8) * (g.W / 8);
    int bps = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_conv_wgrad_tiled<CIN, COUT>, 256, 0);
    long grid = (long)(bps > 0 ? bps : 1) * num_sms;
    if (grid > ntiles) grid = ntiles;
    k_conv_wgrad_tiled<CIN, COUT><<<(unsigned)grid, 256, 0, st>>>(g, in, dout, dw);
}

void conv_wgrad(cudaStream_t st, Geom g, Slice in, int cin, Slice dout, int cout, float *dw, int num_sms) {
    const bool tiled = g.W % 8 == 0 && g.H % 8 == 0 && in.stride % 8 == 0 && in.off % 8 == 0 &&
                       dout.stride % 8 == 0 && dout.off % 8 == 0;
    if (tiled) {
        if (cin == 16 && cout == 16) return wgrad_tiled<16, 16>(st, g, in, dout, dw, num_sms);
        if (cin == 16 && cout == 32) return wgrad_tiled<16, 32>(st, g, in, dout, dw, num_sms);
        if (cin == 32 && cout == 16) return wgrad_tiled<32, 16>(st, g, in, dout, dw, num_sms);
        if (cin == 32 && cout == 32) return wgrad_tiled<32, 32>(st, g, in, dout, dw, num_sms);
        if (cin == 64 && cout == 16) return wgrad_tiled<64, 16>(st, g, in, dout, dw, num_sms);
    }
    const long chunk = 2048;
    const int tiles = 27 * (cout / 16) * (cin / 8);
    dim3 grid((unsigned)((g.voxels() + chunk - 1) / chunk), (unsigned)((tiles + 3) / 4));
    k_conv_wgrad<<<grid, 128, 0, st>>>(g, in, cin, dout, cout, chunk, dw);
}

}  // namespace sg

struct Surrogate {
    Handle *h = nullptr;
    int engine = 1;  // forward and data-gradient convolutions: 0 mma.sync, 1 tcgen05
    int n_solver = 0, factor = 2, m = 0, batch_max = 0;
    double L = 0;
    sg::FeatParams fp{};
    sg::Net net;
    // parameters: fp32 master, bf16 copy, gradient, Adam moments, flipped weights
    float *w32 = nullptr, *g32 = nullptr, *am = nullptr, *av = nullptr;
    __nv_bfloat16 *wb = nullptr, *wflip = nullptr;
    long adam_t = 0;
    // activations (bf16) and their gradients, sized for batch_max
    __nv_bfloat16 *x0 = nullptr, *t0 = nullptr, *c0 = nullptr, *p1 = nullptr, *t1 = nullptr, *c1 = nullptr,
                  *p2 = nullptr, *q2 = nullptr, *u1 = nullptr, *u0 = nullptr;
    __nv_bfloat16 *dt0 = nullptr, *dc0 = nullptr, *dp1 = nullptr, *dt1 = nullptr, *dc1 = nullptr,
                  *dp2 = nullptr, *dq2 = nullptr, *du1 = nullptr, *du0 = nullptr, *dlog = nullptr, *tmp = nullptr;
    float *logits = nullptr, *pred = nullptr, *targ = nullptr, *pw_s = nullptr, *pg_s = nullptr,
          *mask_solver = nullptr, *up_pred = nullptr;
    gbg_sample *dsmp = nullptr;
    double *dloss = nullptr;
    std::vector<void *> owned;
};

namespace {

using sg::Geom;
using sg::Slice;

template <typename T>
T *salloc(Surrogate &s, size_t count) {
    void *p = nullptr;
    if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) return nullptr;
    s.owned.push_back(p);
    return (T *)p;
}

// forward for B samples already featurised in s.x0; logits in s.logits
void forward(Surrogate &s, int B) {
    cudaStream_t st = s.h->stream;
    const int m = s.m;
    Geom g0{B, m, m, m}, g1{B, m / 2, m / 2, m / 2}, g2{B, m / 4, m / 4, m / 4};
    const auto &Ly = s.net.L;
    auto W = [&](int i) { return s.wb + Ly[i].w_off; };
    auto Bi = [&](int i) { return s.w32 + Ly[i].b_off; };
    sg::conv_fwd(st, g0, Slice{s.x0, 16, 0}, 16, W(0), Bi(0), Slice{s.t0, 16, 0}, nullptr, 16, true, s.engine, s.h->num_sms, s.h->dev_status);
    sg::conv_fwd(st, g0, Slice{s.t0, 16, 0}, 16, W(1), Bi(1), Slice{s.c0, 32, 16}, nullptr, 16, true, s.engine, s.h->num_sms, s.h->dev_status);
    sg::k_pool2<<<sg::grid_n(g1.voxels() * 16), 256, 0, st>>>(g1, 16, Slice{s.c0, 32, 16}, Slice{s.p1, 16, 0});
    sg::conv_fwd(st, g1, Slice{s.p1, 16, 0}, 16, W(2), Bi(2), Slice{s.t1, 32, 0}, nullptr, 32, true, s.engine, s.h->num_sms, s.h->dev_status);
    sg::conv_fwd(st, g1, Slice{s.t1, 32, 0}, 32, W(3), Bi(3), Slice{s.c1, 64, 32}, nullptr, 32, true, s.engine, s.h->num_sms, s.h->dev_status);
    sg::k_pool2<<<sg::grid_n(g2.voxels() * 32), 256, 0, st>>>(g2, 32, Slice{s.c1, 64, 32}, Slice{s.p2, 32, 0});
    sg::conv_fwd(st, g2, Slice{s.p2, 32, 0}, 32, W(4), Bi(4), Slice{s.q2, 32, 0}, nullptr, 32, true, s.engine, s.h->num_sms, s.h->dev_status);
    sg::k_up2<<<sg::grid_n(g1.voxels() * 32), 256, 0, st>>>(g1, 32, Slice{s.q2, 32, 0}, Slice{s.c1, 64, 0});
    sg::conv_fwd(st, g1, Slice{s.c1, 64, 0}, 64, W(5), Bi(5), Slice{s.u1, 16, 0}, nullptr, 16, true, s.engine, s.h->num_sms, s.h->dev_status);
    sg::k_up2<<<sg::grid_n(g0.voxels() * 16), 256, 0, st>>>(g0, 16, Slice{s.u1, 16, 0}, Slice{s.c0, 32, 0});
    sg::conv_fwd(st, g0, Slice{s.c0, 32, 0}, 32, W(6), Bi(6), Slice{s.u0, 16, 0}, nullptr, 16, true, s.engine, s.h->num_sms, s.h->dev_status);
    sg::conv_fwd(st, g0, Slice{s.u0, 16, 0}, 16, W(7), Bi(7), Slice{nullptr, 0, 0}, s.logits, 16, false, s.engine, s.h->num_sms, s.h->dev_status);
    s.h->launches += 12;
}

// data gradient of layer i: din (cin channels) from dout (cout channels)
void data_grad(Surrogate &s, Geom g, int i, Slice dout, Slice din) {
    const auto &l = s.net.L[i];
    const long n = (long)l.cout * 27 * l.cin;
    sg::k_flip_weights<<<sg::grid_n(n), 256, 0, s.h->stream>>>(s.wb + l.w_off, l.cout, l.cin, s.wflip);
    sg::conv_fwd(s.h->stream, g, dout, l.cout, s.wflip, nullptr, din, nullptr, l.cin, false, s.engine, s.h->num_sms,
                 s.h->dev_status);
    s.h->launches += 2;
}

void param_grad(Surrogate &s, Geom g, int i, Slice in, Slice dout) {
    const auto &l = s.net.L[i];
    sg::conv_wgrad(s.h->stream, g, in, l.cin, dout, l.cout, s.g32 + l.w_off, s.h->num_sms);
    dim3 gb(64, l.cout);
    sg::k_bias_grad<<<gb, 256, 0, s.h->stream>>>(g.voxels(), l.cout, dout, s.g32 + l.b_off);
    s.h->launches += 2;
}

void relu_bwd(Surrogate &s, Geom g, int C, Slice y, Slice dy) {
    sg::k_relu_bwd<<<sg::grid_n(g.voxels() * C), 256, 0, s.h->stream>>>(g.voxels(), C, y, dy);
    s.h->launches++;
}

// accumulate src slice into dst slice (bf16, fp32 add)
__global__ void k_add_slice(long nv, int C, Slice src, Slice dst) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nv * C; i += (long)gridDim.x * blockDim.x) {
        const long v = i / C;
        const int c = (int)(i % C);
        __nv_bfloat16 &d = dst.p[v * dst.stride + dst.off + c];
        d = __float2bfloat16(__bfloat162float(d) + __bfloat162float(src.p[v * src.stride + src.off + c]));
    }
}

// backward from s.dlog (bf16 [voxels][16], channel 0 nonzero); gradients into s.g32
void backward(Surrogate &s, int B) {
    cudaStream_t st = s.h->stream;
    const int m = s.m;
    Geom g0{B, m, m, m}, g1{B, m / 2, m / 2, m / 2}, g2{B, m / 4, m / 4, m / 4};
    // out
    param_grad(s, g0, 7, Slice{s.u0, 16, 0}, Slice{s.dlog, 16, 0});
    data_grad(s, g0, 7, Slice{s.dlog, 16, 0}, Slice{s.du0, 16, 0});
    // d0
    relu_bwd(s, g0, 16, Slice{s.u0, 16, 0}, Slice{s.du0, 16, 0});
    param_grad(s, g0, 6, Slice{s.c0, 32, 0}, Slice{s.du0, 16, 0});
    data_grad(s, g0, 6, Slice{s.du0, 16, 0}, Slice{s.dc0, 32, 0});
    // up -> u1
    sg::k_up2_bwd<<<sg::grid_n(g1.voxels() * 16), 256, 0, st>>>(g1, 16, Slice{s.dc0, 32, 0}, Slice{s.du1, 16, 0});
    // d1
    relu_bwd(s, g1, 16, Slice{s.u1, 16, 0}, Slice{s.du1, 16, 0});
    param_grad(s, g1, 5, Slice{s.c1, 64, 0}, Slice{s.du1, 16, 0});
    data_grad(s, g1, 5, Slice{s.du1, 16, 0}, Slice{s.dc1, 64, 0});
    // up -> q2
    sg::k_up2_bwd<<<sg::grid_n(g2.voxels() * 32), 256, 0, st>>>(g2, 32, Slice{s.dc1, 64, 0}, Slice{s.dq2, 32, 0});
    // mid
    relu_bwd(s, g2, 32, Slice{s.q2, 32, 0}, Slice{s.dq2, 32, 0});
    param_grad(s, g2, 4, Slice{s.p2, 32, 0}, Slice{s.dq2, 32, 0});
    data_grad(s, g2, 4, Slice{s.dq2, 32, 0}, Slice{s.dp2, 32, 0});
    // pool -> c1[32:64], added to d1's gradient there
    sg::k_pool2_bwd<<<sg::grid_n(g1.voxels() * 32), 256, 0, st>>>(g1, 32, Slice{s.dp2, 32, 0}, Slice{s.tmp, 32, 0});
    k_add_slice<<<sg::grid_n(g1.voxels() * 32), 256, 0, st>>>(g1.voxels(), 32, Slice{s.tmp, 32, 0}, Slice{s.dc1, 64, 32});
    // e1b
    relu_bwd(s, g1, 32, Slice{s.c1, 64, 32}, Slice{s.dc1, 64, 32});
    param_grad(s, g1, 3, Slice{s.t1, 32, 0}, Slice{s.dc1, 64, 32});
    data_grad(s, g1, 3, Slice{s.dc1, 64, 32}, Slice{s.dt1, 32, 0});
    // e1a
    relu_bwd(s, g1, 32, Slice{s.t1, 32, 0}, Slice{s.dt1, 32, 0});
    param_grad(s, g1, 2, Slice{s.p1, 16, 0}, Slice{s.dt1, 32, 0});
    data_grad(s, g1, 2, Slice{s.dt1, 32, 0}, Slice{s.dp1, 16, 0});
    // pool -> c0[16:32], added to d0's gradient there
    sg::k_pool2_bwd<<<sg::grid_n(g0.voxels() * 16), 256, 0, st>>>(g0, 16, Slice{s.dp1, 16, 0}, Slice{s.tmp, 16, 0});
    k_add_slice<<<sg::grid_n(g0.voxels() * 16), 256, 0, st>>>(g0.voxels(), 16, Slice{s.tmp, 16, 0}, Slice{s.dc0, 32, 16});
    // e0b
    relu_bwd(s, g0, 16, Slice{s.c0, 32, 16}, Slice{s.dc0, 32, 16});
    param_grad(s, g0, 1, Slice{s.t0, 16, 0}, Slice{s.dc0, 32, 16});
    data_grad(s, g0, 1, Slice{s.dc0, 32, 16}, Slice{s.dt0, 16, 0});
    // e0a
    relu_bwd(s, g0, 16, Slice{s.t0, 16, 0}, Slice{s.dt0, 16, 0});
    param_grad(s, g0, 0, Slice{s.x0, 16, 0}, Slice{s.dt0, 16, 0});
    s.h->launches += 6;
}

// dlogit buffer: channel 0 from the loss, the other 15 channels zero
__global__ void k_scatter_dlogit(long nv, const __nv_bfloat16 *__restrict__ d0, __nv_bfloat16 *__restrict__ d16) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nv * 16; i += (long)gridDim.x * blockDim.x)
        d16[i] = (i % 16 == 0) ? d0[i / 16] : __float2bfloat16(0.f);
}

__global__ void k_channel0(long nv, const float *__restrict__ l16, float *__restrict__ l1) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nv; i += (long)gridDim.x * blockDim.x) l1[i] = l16[i * 16];
}

void featurise(Surrogate &s, const gbg_sample *dsamples, int B) {
    sg::k_features<<<sg::grid_n((long)B * s.m * s.m * s.m), 256, 0, s.h->stream>>>(B, s.m, s.factor, dsamples, s.pw_s,
                                                                                   s.pg_s, s.fp, s.x0);
    s.h->launches++;
}

// loss (and, with targets, dlogit) for the B samples in the forward buffers
int loss_and_backward(Surrogate &s, int B, const float *targets, bool grad, double *loss) {
    cudaStream_t st = s.h->stream;
    const long nv = (long)B * s.m * s.m * s.m;
    float *l1 = s.pred;  // reuse: channel-0 logits, then predictions
    k_channel0<<<sg::grid_n(nv), 256, 0, st>>>(nv, s.logits, l1);
    GBG_CUDA_TRY(cudaMemsetAsync(s.dloss, 0, sizeof(double), st));
    sg::k_loss<<<sg::grid_n(nv, 1024), 256, 0, st>>>(nv, l1, targets, s.pred, grad ? s.tmp : nullptr, 1.f, s.dloss);
    s.h->launches += 2;
    if (grad) {
        k_scatter_dlogit<<<sg::grid_n(nv * 16), 256, 0, st>>>(nv, s.tmp, s.dlog);
        GBG_CUDA_TRY(cudaMemsetAsync(s.g32, 0, s.net.nparams * sizeof(float), st));
        backward(s, B);
        s.h->launches++;
    }
    if (loss) {
        GBG_CUDA_TRY(cudaMemcpyAsync(loss, s.dloss, sizeof(double), cudaMemcpyDeviceToHost, st));
        GBG_CUDA_TRY(cudaStreamSynchronize(st));
    }
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
}

}  // namespace

int surrogate_create(Handle &h, const gbg_surrogate_config &c, Surrogate **out) {
    if (c.factor != 2 || h.n % 8 != 0 || c.batch_max < 1) {
        set_error("surrogate: factor must be 2, n a multiple of 8, batch_max >= 1");
        return GBG_ERR_UNSUPPORTED;
    }
    Surrogate *s = new Surrogate();
    s->h = &h;
    s->n_solver = h.n;
    s->factor = c.factor;
    s->m = h.n / c.factor;
    s->batch_max = c.batch_max;
    s->L = c.L;
    s->fp = sg::FeatParams{c.dw_lo, c.dw_hi, c.rho_lo, c.rho_hi, c.t_lo, c.t_hi, c.L, (double)h.n, 1.5};
    const long P = s->net.nparams;
    const long v0 = (long)c.batch_max * s->m * s->m * s->m, v1 = v0 / 8, v2 = v0 / 64;
    const size_t N = h.N;
    bool ok = (s->w32 = salloc<float>(*s, P)) && (s->g32 = salloc<float>(*s, P)) && (s->am = salloc<float>(*s, P)) &&
              (s->av = salloc<float>(*s, P)) && (s->wb = salloc<__nv_bfloat16>(*s, P)) &&
              (s->wflip = salloc<__nv_bfloat16>(*s, 64L * 27 * 64)) &&
              (s->x0 = salloc<__nv_bfloat16>(*s, v0 * 16)) && (s->t0 = salloc<__nv_bfloat16>(*s, v0 * 16)) &&
              (s->c0 = salloc<__nv_bfloat16>(*s, v0 * 32)) && (s->p1 = salloc<__nv_bfloat16>(*s, v1 * 16)) &&
              (s->t1 = salloc<__nv_bfloat16>(*s, v1 * 32)) && (s->c1 = salloc<__nv_bfloat16>(*s, v1 * 64)) &&
              (s->p2 = salloc<__nv_bfloat16>(*s, v2 * 32)) && (s->q2 = salloc<__nv_bfloat16>(*s, v2 * 32)) &&
              (s->u1 = salloc<__nv_bfloat16>(*s, v1 * 16)) && (s->u0 = salloc<__nv_bfloat16>(*s, v0 * 16)) &&
              (s->dt0 = salloc<__nv_bfloat16>(*s, v0 * 16)) && (s->dc0 = salloc<__nv_bfloat16>(*s, v0 * 32)) &&
              (s->dp1 = salloc<__nv_bfloat16>(*s, v1 * 16)) && (s->dt1 = salloc<__nv_bfloat16>(*s, v1 * 32)) &&
              (s->dc1 = salloc<__nv_bfloat16>(*s, v1 * 64)) && (s->dp2 = salloc<__nv_bfloat16>(*s, v2 * 32)) &&
              (s->dq2 = salloc<__nv_bfloat16>(*s, v2 * 32)) && (s->du1 = salloc<__nv_bfloat16>(*s, v1 * 16)) &&
              (s->du0 = salloc<__nv_bfloat16>(*s, v0 * 16)) && (s->dlog = salloc<__nv_bfloat16>(*s, v0 * 16)) &&
              (s->tmp = salloc<__nv_bfloat16>(*s, v0 * 32)) && (s->logits = salloc<float>(*s, v0 * 16)) &&
              (s->pred = salloc<float>(*s, v0)) && (s->pw_s = salloc<float>(*s, (size_t)s->m * s->m * s->m)) &&
              (s->pg_s = salloc<float>(*s, (size_t)s->m * s->m * s->m)) && (s->mask_solver = salloc<float>(*s, N)) &&
              (s->up_pred = salloc<float>(*s, (size_t)c.batch_max * N)) &&
              (s->dsmp = salloc<gbg_sample>(*s, c.batch_max)) && (s->dloss = salloc<double>(*s, 1));
    if (!ok) {
        for (void *p : s->owned) cudaFree(p);
        delete s;
        set_error("surrogate: device allocation failed");
        return GBG_ERR_NOMEM;
    }
    // anatomy on the surrogate grid (averaged) and the solver's tissue mask
    {
        std::vector<double> pw(N), pg(N);
        cudaMemcpy(pw.data(), h.pw, N * sizeof(double), cudaMemcpyDeviceToHost);
        cudaMemcpy(pg.data(), h.pg, N * sizeof(double), cudaMemcpyDeviceToHost);
        const int n = h.n, m = s->m, f = c.factor;
        std::vector<float> aw((size_t)m * m * m, 0.f), ag(aw.size(), 0.f), mk(N);
        for (int z = 0; z < n; ++z)
            for (int y = 0; y < n; ++y)
                for (int x = 0; x < n; ++x) {
                    const size_t g = (size_t)x + (size_t)n * ((size_t)y + (size_t)n * z);
                    const size_t q = (size_t)(x / f) + (size_t)m * ((size_t)(y / f) + (size_t)m * (z / f));
                    aw[q] += (float)(pw[g] / (f * f * f));
                    ag[q] += (float)(pg[g] / (f * f * f));
                    mk[g] = pw[g] + pg[g] > 0 ? 1.f : 0.f;
                }
        cudaMemcpy(s->pw_s, aw.data(), aw.size() * sizeof(float), cudaMemcpyHostToDevice);
        cudaMemcpy(s->pg_s, ag.data(), ag.size() * sizeof(float), cudaMemcpyHostToDevice);
        cudaMemcpy(s->mask_solver, mk.data(), N * sizeof(float), cudaMemcpyHostToDevice);
    }
    // He-normal initial weights from a fixed seed, zero biases except the
    // output logit's, which starts at -4 (sigmoid 0.018: most of the brain
    // holds no tumour, so training starts near the typical density)
    {
        std::vector<float> w(P, 0.f);
        unsigned long long st = 0x9E3779B97F4A7C15ull ^ (unsigned long long)c.seed;
        auto uni = [&]() {
            st = st * 6364136223846793005ull + 1442695040888963407ull;
            return ((st >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        };
        for (const auto &l : s->net.L) {
            const double sd = std::sqrt(2.0 / (27.0 * l.cin));
            for (long i = 0; i < (long)l.cout * 27 * l.cin; ++i) {
                const double u1 = uni(), u2 = uni();
                w[l.w_off + i] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
            }
        }
        w[s->net.L.back().b_off] = -4.f;
        cudaMemcpy(s->w32, w.data(), P * sizeof(float), cudaMemcpyHostToDevice);
        cudaMemset(s->am, 0, P * sizeof(float));
        cudaMemset(s->av, 0, P * sizeof(float));
        sg::k_f32_to_bf16<<<sg::grid_n(P), 256>>>(P, s->w32, s->wb);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) {
        for (void *p : s->owned) cudaFree(p);
        delete s;
        set_error("surrogate: initialisation failed");
        return GBG_ERR_CUDA;
    }
    *out = s;
    return GBG_OK;
}

void surrogate_destroy(Surrogate *s) {
    if (!s) return;
    cudaStreamSynchronize(s->h->stream);
    for (void *p : s->owned) cudaFree(p);
    delete s;
}

long surrogate_nparams(const Surrogate &s) { return s.net.nparams; }
int surrogate_batch_max(const Surrogate &s) { return s.batch_max; }
int surrogate_set_engine(Surrogate &s, int engine) {
    if (engine != 0 && engine != 1) {
        set_error("convolution engine: 0 (mma.sync) or 1 (tcgen05)");
        return GBG_ERR_ARG;
    }
    s.engine = engine;
    return GBG_OK;
}
const float *surrogate_prediction(const Surrogate &s) { return s.up_pred; }

int surrogate_get_params(Surrogate &s, float *out) {
    GBG_CUDA_TRY(cudaMemcpy(out, s.w32, s.net.nparams * sizeof(float), cudaMemcpyDeviceToHost));
    return GBG_OK;
}

int surrogate_set_params(Surrogate &s, const float *in) {
    GBG_CUDA_TRY(cudaMemcpy(s.w32, in, s.net.nparams * sizeof(float), cudaMemcpyHostToDevice));
    sg::k_f32_to_bf16<<<sg::grid_n(s.net.nparams), 256, 0, s.h->stream>>>(s.net.nparams, s.w32, s.wb);
    GBG_CUDA_TRY(cudaStreamSynchronize(s.h->stream));
    return GBG_OK;
}

// loss and flat gradient of a batch against host targets (surrogate grid, fp32)
int surrogate_loss_grad(Surrogate &s, const gbg_sample *samples, int B, const float *targets_host, double *loss,
                        float *grad_host) {
    cudaStream_t st = s.h->stream;
    const size_t M = (size_t)s.m * s.m * s.m;
    GBG_CUDA_TRY(cudaMemcpyAsync(s.dsmp, samples, B * sizeof(gbg_sample), cudaMemcpyHostToDevice, st));
    float *targ = (float *)s.up_pred;  // scratch large enough for B surrogate fields
    GBG_CUDA_TRY(cudaMemcpyAsync(targ, targets_host, B * M * sizeof(float), cudaMemcpyHostToDevice, st));
    featurise(s, s.dsmp, B);
    forward(s, B);
    if (int rc = loss_and_backward(s, B, targ, grad_host != nullptr, loss)) return rc;
    if (grad_host) {
        GBG_CUDA_TRY(cudaMemcpyAsync(grad_host, s.g32, s.net.nparams * sizeof(float), cudaMemcpyDeviceToHost, st));
        GBG_CUDA_TRY(cudaStreamSynchronize(st));
    }
    return check_device_status(*s.h);
}

// features of B samples (host copy, [B][m^3][16] as float) for the oracle
int surrogate_features(Surrogate &s, const gbg_sample *samples, int B, float *out) {
    cudaStream_t st = s.h->stream;
    const size_t M = (size_t)s.m * s.m * s.m;
    GBG_CUDA_TRY(cudaMemcpyAsync(s.dsmp, samples, B * sizeof(gbg_sample), cudaMemcpyHostToDevice, st));
    featurise(s, s.dsmp, B);
    std::vector<__nv_bfloat16> tmp((size_t)B * M * 16);
    GBG_CUDA_TRY(cudaMemcpyAsync(tmp.data(), s.x0, tmp.size() * 2, cudaMemcpyDeviceToHost, st));
    GBG_CUDA_TRY(cudaStreamSynchronize(st));
    for (size_t i = 0; i < tmp.size(); ++i) out[i] = __bfloat162float(tmp[i]);
    return GBG_OK;
}

// train on S samples: targets from the handle's batched solver (final densities
// averaged onto the surrogate grid), then `epochs` passes of Adam in batches
int surrogate_train(Surrogate &s, const gbg_sample *samples, int S, int epochs, int batch, double lr,
                    unsigned long long seed, double *loss_out) {
    Handle &h = *s.h;
    cudaStream_t st = h.stream;
    const size_t M = (size_t)s.m * s.m * s.m;
    if (batch < 1 || batch > s.batch_max || S < batch) {
        set_error("surrogate_train: need 1 <= batch <= batch_max and S >= batch");
        return GBG_ERR_ARG;
    }
    float *targets = nullptr;
    GBG_CUDA_TRY(cudaMalloc((void **)&targets, (size_t)S * M * sizeof(float)));
    // training targets, in chunks of the handle's population capacity
    gbg_sample *dsm = batch_samples(h);
    int rc = GBG_OK;
    gbg_batch_opts o{s.L, 0.1, 1.0, 0, 0.0};
    for (int s0 = 0; s0 < S && rc == GBG_OK; s0 += h.max_samples) {
        const int cnt = std::min(h.max_samples, S - s0);
        if (cudaMemcpyAsync(dsm, samples + s0, cnt * sizeof(gbg_sample), cudaMemcpyHostToDevice, st) != cudaSuccess) {
            rc = GBG_ERR_CUDA;
            break;
        }
        std::vector<long> steps(cnt);
        rc = batch_solve_device(h, dsm, cnt, o, nullptr, steps.data());
        if (rc) break;
        rc = check_device_status(h);
        if (rc) break;
        // final fields sit in buffer (nsteps & 1); average each onto the surrogate grid
        for (int k = 0; k < cnt; ++k) {
            const float *src = h.bphi[steps[k] & 1] + (size_t)k * h.N;
            sg::k_down2_f32<<<sg::grid_n(M), 256, 0, st>>>(1, h.n, src, targets + (size_t)(s0 + k) * M);
        }
        h.launches += cnt;
    }
    // Adam over shuffled batches
    std::vector<int> order(S);
    for (int i = 0; i < S; ++i) order[i] = i;
    unsigned long long rs = seed * 2862933555777941757ull + 3037000493ull;
    auto rnd = [&]() {
        rs = rs * 6364136223846793005ull + 1442695040888963407ull;
        return (unsigned)(rs >> 33);
    };
    std::vector<gbg_sample> bs(batch);
    double last = 0;
    float *btarg = (float *)s.up_pred;
    for (int ep = 0; ep < epochs && rc == GBG_OK; ++ep) {
        for (int i = S - 1; i > 0; --i) std::swap(order[i], order[rnd() % (i + 1)]);
        double sum = 0;
        int nb = 0;
        for (int b0 = 0; b0 + batch <= S && rc == GBG_OK; b0 += batch) {
            for (int k = 0; k < batch; ++k) {
                bs[k] = samples[order[b0 + k]];
                if (cudaMemcpyAsync(btarg + (size_t)k * M, targets + (size_t)order[b0 + k] * M, M * sizeof(float),
                                    cudaMemcpyDeviceToDevice, st) != cudaSuccess)
                    rc = GBG_ERR_CUDA;
            }
            if (cudaMemcpyAsync(s.dsmp, bs.data(), batch * sizeof(gbg_sample), cudaMemcpyHostToDevice, st) != cudaSuccess)
                rc = GBG_ERR_CUDA;
            if (rc) break;
            featurise(s, s.dsmp, batch);
            forward(s, batch);
            double l = 0;
            rc = loss_and_backward(s, batch, btarg, true, &l);
            if (rc) break;
            ++s.adam_t;
            const float b1 = 0.9f, b2 = 0.999f;
            const float c1 = 1.f - (float)std::pow(b1, (double)s.adam_t), c2 = 1.f - (float)std::pow(b2, (double)s.adam_t);
            // linear learning-rate warm-up over the first 100 updates of the
            // network's life: large early Adam steps switch ReLUs off for good
            const double lr_t = lr * std::min(1.0, (double)s.adam_t / 100.0);
            sg::k_adam<<<sg::grid_n(s.net.nparams), 256, 0, st>>>(s.net.nparams, s.w32, s.g32, s.am, s.av, s.wb,
                                                                   (float)lr_t, b1, b2, 1e-8f, c1, c2, 1.f);
            h.launches++;
            sum += l;
            ++nb;
        }
        last = nb ? sum / nb : 0;
    }
    cudaFree(targets);
    if (rc) return rc;
    GBG_CUDA_TRY(cudaGetLastError());
    if (int st_rc = check_device_status(h)) return st_rc;
    if (loss_out) *loss_out = last;
    return GBG_OK;
}

// predicted final densities of B samples on the solver grid (nearest 2x
// upsampling of the surrogate field, zero off tissue) into s.up_pred, and
// optionally their log-likelihoods (device results)
int surrogate_predict(Surrogate &s, const gbg_sample *samples_device, int B, gbg_lik_result *lik_device) {
    cudaStream_t st = s.h->stream;
    const long nv = (long)B * s.m * s.m * s.m;
    featurise(s, samples_device, B);
    forward(s, B);
    k_channel0<<<sg::grid_n(nv), 256, 0, st>>>(nv, s.logits, s.pred);
    sg::k_loss<<<sg::grid_n(nv, 1024), 256, 0, st>>>(nv, s.pred, nullptr, s.pred, nullptr, 1.f, nullptr);
    sg::k_up2_f32<<<sg::grid_n((long)B * s.h->N), 256, 0, st>>>(B, s.m, s.pred, s.mask_solver, s.up_pred);
    s.h->launches += 3;
    GBG_CUDA_TRY(cudaGetLastError());
    if (lik_device) return lik_evaluate(*s.h, s.up_pred, nullptr, B, lik_device);
    return GBG_OK;
}

}  // namespace gbg
