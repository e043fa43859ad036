// Imaging log-likelihood of HGG_Likelihood (source/Likelihood/source/HGG_Likelihood.cpp),
// as a gather-and-reduce over compact observation lists:
//   PET term  (:40-75)   over voxels with ix,iy,iz = 0 mod stepPet and PET > 0:
//             -0.5 N log(2 pi sigma^2) - 0.5/sigma^2 * sum (u - scale*PET)^2
//   T1/T2     (:77-128)  over the Sphere.dat points with coordinates = 0 mod
//             stepTi (or every voxel): sum of log Bernoulli(alpha(u)) with
//             alpha = 0.5 + 0.5 sgn(u - uc) (1 - exp(-(u - uc)^2 / slope))
//             (:136-160)
// The lists are built once per observation set on the host. Per sample, each
// CTA reduces a chunk of both lists with warp shuffles into three double
// partial sums (scratch), and a second pass adds a sample's partials in a
// fixed order, so results are deterministic. Accumulation is double (the
// reference's is long double).
//
// Compiled with -fmad=false: (u - scale*PET)^2 and the exponent round as the
// reference's plain double expressions do.
#include <mutex>
#include <vector>

#include "gbg_internal.cuh"
#include "lik_terms.cuh"

namespace gbg {

namespace {

constexpr int kLikThreads = 256;
constexpr int kLikPerThread = 8;
constexpr int kLikChunk = kLikThreads * kLikPerThread;

struct LikArgs {
    int n_pet, n_ti, chunks;
    const int *pet_idx;
    const double *pet_val;
    const int *ti_idx;
    const double *t1_val, *t2_val;
    double pet_scale, t1_uc, t2_uc, is2;
    size_t stride;
    double *partials;  // [S][chunks][3]
};

// phi of sample s: F32 buffers chosen per sample by its step parity, or one
// double / float field array at stride.
struct PhiSource {
    const float *f0, *f1;       // population buffers (f1 may equal f0)
    const double *d;            // double fields (exact FP64 mode)
    const SampleRec *recs;      // if non-null, buffer = recs[s].nsteps & 1
    __device__ __forceinline__ double at(int s, size_t stride, int c) const {
        if (d) return d[(size_t)s * stride + c];
        const float *b = (recs && (recs[s].nsteps & 1)) ? f1 : f0;
        return (double)b[(size_t)s * stride + c];
    }
    __device__ __forceinline__ double pet(const LikArgs &a, int s, int i) const {
        return at(s, a.stride, a.pet_idx[i]);
    }
    __device__ __forceinline__ double ti(const LikArgs &a, int s, int i) const {
        return at(s, a.stride, a.ti_idx[i]);
    }
};

// phi of affine model s at the i-th entry of an observation list, from the
// model gathered at the list's cells: cols = [pet block | ti block], each
// block (P + 2) rows of its list's length: phi0, J_0 .. J_{P-1}, tissue mask.
// The same float operations as forming the whole field would do:
// v = phi0; v = fma(delta_p, J_p, v) for p = 0..P-1; clamp to [0, 1]; 0
// outside the mask.
struct AffineSource {
    const float *pet_cols, *ti_cols;
    const double *delta;
    int P;
    __device__ __forceinline__ double eval(const float *cols, int len, int s, int i) const {
        float v = cols[i];
        for (int p = 0; p < P; ++p) v = fmaf((float)delta[(size_t)s * P + p], cols[(size_t)(1 + p) * len + i], v);
        v = fminf(fmaxf(v, 0.f), 1.f);
        return cols[(size_t)(P + 1) * len + i] != 0.f ? (double)v : 0.0;
    }
    __device__ __forceinline__ double pet(const LikArgs &a, int s, int i) const {
        return eval(pet_cols, a.n_pet, s, i);
    }
    __device__ __forceinline__ double ti(const LikArgs &a, int s, int i) const {
        return eval(ti_cols, a.n_ti, s, i);
    }
};

template <class Src>
__global__ void __launch_bounds__(kLikThreads) k_lik_partial(LikArgs a, Src src) {
    const int s = blockIdx.y;
    const int chunk = blockIdx.x;
    double sp = 0.0, s1 = 0.0, s2 = 0.0;
    const int base = chunk * kLikChunk;
    for (int k = 0; k < kLikPerThread; ++k) {
        const int i = base + k * kLikThreads + threadIdx.x;
        if (i < a.n_pet) {
            const double u = src.pet(a, s, i);
            const double pv = a.pet_val[i];
            const double r = u - a.pet_scale * pv;
            sp += r * r;
        }
        if (i < a.n_ti) {
            const double u = src.ti(a, s, i);
            s1 += log_bernoulli(u, a.t1_val[i], a.t1_uc, a.is2);
            s2 += log_bernoulli(u, a.t2_val[i], a.t2_uc, a.is2);
        }
    }
    sp = warp_sum(sp);
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    __shared__ double red[3][kLikThreads / 32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        red[0][w] = sp;
        red[1][w] = s1;
        red[2][w] = s2;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int j = 0; j < kLikThreads / 32; ++j) t += red[threadIdx.x][j];
        a.partials[((size_t)s * a.chunks + chunk) * 3 + threadIdx.x] = t;
    }
}

__global__ void k_lik_final(const double *__restrict__ partials, int chunks, int S, int n_pet,
                            double pet_sigma2, gbg_lik_result *__restrict__ out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    double sp = 0.0, s1 = 0.0, s2 = 0.0;
    for (int c = 0; c < chunks; ++c) {
        const double *p = partials + ((size_t)s * chunks + c) * 3;
        sp += p[0];
        s1 += p[1];
        s2 += p[2];
    }
    // :70-74
    const double p1 = -0.5 * n_pet * log(2. * 3.14159265358979323846 * pet_sigma2);
    const double p2 = -0.5 * (1. / pet_sigma2) * sp;
    gbg_lik_result r;
    r.l_pet = p1 + p2;
    r.l_t1 = s1;
    r.l_t2 = s2;
    r.total = r.l_pet + r.l_t1 + r.l_t2;
    r.n_pet = n_pet;
    out[s] = r;
}

template <typename T>
int upload(T **dst, const std::vector<T> &v) {
    if (*dst) {
        cudaFree(*dst);
        *dst = nullptr;
    }
    if (v.empty()) return GBG_OK;
    GBG_CUDA_TRY(cudaMalloc((void **)dst, v.size() * sizeof(T)));
    GBG_CUDA_TRY(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return GBG_OK;
}

template <class Src>
int run_lik(Handle &h, const Src &src, int S, gbg_lik_result *out_device) {
    if (!h.obs.valid) {
        set_error("observations not set");
        return GBG_ERR_STATE;
    }
    if (int rc = lik_reserve(h, S)) return rc;
    const int items = h.obs.n_pet > h.obs.n_ti ? h.obs.n_pet : h.obs.n_ti;
    const int chunks = items > 0 ? (items + kLikChunk - 1) / kLikChunk : 1;
    LikArgs a;
    a.n_pet = h.obs.n_pet;
    a.n_ti = h.obs.n_ti;
    a.chunks = chunks;
    a.pet_idx = h.obs.pet_idx;
    a.pet_val = h.obs.pet_val;
    a.ti_idx = h.obs.ti_idx;
    a.t1_val = h.obs.t1_val;
    a.t2_val = h.obs.t2_val;
    a.pet_scale = h.obs.pet_scale;
    a.t1_uc = h.obs.t1_uc;
    a.t2_uc = h.obs.t2_uc;
    a.is2 = 1. / h.obs.slope;
    a.stride = h.N;
    a.partials = h.lik_partials;
    k_lik_partial<<<dim3(chunks, S), kLikThreads, 0, h.stream>>>(a, src);
    k_lik_final<<<(S + 127) / 128, 128, 0, h.stream>>>(h.lik_partials, chunks, S, h.obs.n_pet,
                                                       h.obs.pet_sigma2, out_device);
    h.launches += 2;
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
}

}  // namespace

// Partial-sum storage of the likelihood reduction for S samples.
int lik_reserve(Handle &h, int S) {
    const int items = h.obs.n_pet > h.obs.n_ti ? h.obs.n_pet : h.obs.n_ti;
    const int chunks = items > 0 ? (items + kLikChunk - 1) / kLikChunk : 1;
    const size_t need = (size_t)S * chunks * 3;
    if (need > h.lik_partials_cap) {
        ++h.state_gen;
        if (h.lik_partials) cudaFree(h.lik_partials);
        h.lik_partials = nullptr;
        h.lik_partials_cap = 0;
        GBG_CUDA_TRY(cudaMalloc((void **)&h.lik_partials, need * sizeof(double)));
        h.lik_partials_cap = need;
    }
    return GBG_OK;
}


int lik_set_observations(Handle &h, const double *pet, const double *t1, const double *t2,
                         const double *points, long npoints, const gbg_lik_params &p) {
    const int n = h.n;
    if (p.step_pet <= 0 || p.step_ti <= 0 || !(p.pet_sigma2 > 0) || !(p.slope > 0)) {
        set_error("likelihood parameters out of range");
        return GBG_ERR_ARG;
    }
    ++h.state_gen;  // captured batched solves name the observation lists
    std::vector<int> pet_idx, ti_idx;
    std::vector<double> pet_val, v1, v2;
    for (int iz = 0; iz < n; iz++)
        for (int iy = 0; iy < n; iy++)
            for (int ix = 0; ix < n; ix++)
                if ((ix % p.step_pet == 0) && (iy % p.step_pet == 0) && (iz % p.step_pet == 0)) {
                    const size_t g = (size_t)ix + (size_t)n * ((size_t)iy + (size_t)n * iz);
                    if (pet[g] > 0.) {
                        pet_idx.push_back((int)g);
                        pet_val.push_back(pet[g]);
                    }
                }
    if (p.selective) {
        for (long i = 0; i < npoints; i++) {
            // Points(i,0..2) read as int as the reference does (:113-115)
            const int ix = (int)points[i], iy = (int)points[i + npoints], iz = (int)points[i + 2 * npoints];
            if (ix < 0 || iy < 0 || iz < 0 || ix >= n || iy >= n || iz >= n) {
                set_error("point outside the grid");
                return GBG_ERR_ARG;
            }
            if ((ix % p.step_ti == 0) && (iy % p.step_ti == 0) && (iz % p.step_ti == 0)) {
                const size_t g = (size_t)ix + (size_t)n * ((size_t)iy + (size_t)n * iz);
                ti_idx.push_back((int)g);
                v1.push_back(t1[g]);
                v2.push_back(t2[g]);
            }
        }
    } else {
        for (size_t g = 0; g < h.N; ++g) {
            ti_idx.push_back((int)g);
            v1.push_back(t1[g]);
            v2.push_back(t2[g]);
        }
    }
    ObsDevice &o = h.obs;
    o.valid = false;
    int rc;
    if ((rc = upload(&o.pet_idx, pet_idx)) || (rc = upload(&o.pet_val, pet_val)) ||
        (rc = upload(&o.ti_idx, ti_idx)) || (rc = upload(&o.t1_val, v1)) || (rc = upload(&o.t2_val, v2)))
        return rc;
    o.n_pet = (int)pet_idx.size();
    o.n_ti = (int)ti_idx.size();
    o.pet_sigma2 = p.pet_sigma2;
    o.pet_scale = p.pet_scale;
    o.t1_uc = p.t1_uc;
    o.t2_uc = p.t2_uc;
    o.slope = p.slope;
    o.valid = true;
    h.aff_cols_stale = true;
    return GBG_OK;
}

int lik_evaluate(Handle &h, const float *phi_f32, const double *phi_f64, int S,
                 gbg_lik_result *out_device) {
    PhiSource src{phi_f32, phi_f32, phi_f64, nullptr};
    return run_lik(h, src, S, out_device);
}

int lik_evaluate_affine(Handle &h, const float *cols, int P, const double *delta_device, int B,
                        gbg_lik_result *out_device) {
    AffineSource src{cols, cols + (size_t)(P + 2) * h.obs.n_pet, delta_device, P};
    return run_lik(h, src, B, out_device);
}

int lik_evaluate_population(Handle &h, const float *buf0, const float *buf1,
                            const SampleRec *recs_unsorted, int S, gbg_lik_result *out_device) {
    PhiSource src{buf0, buf1, nullptr, recs_unsorted};
    return run_lik(h, src, S, out_device);
}

}  // namespace gbg

// ---- gbg_loglik_noalloc: the same reduction with library-owned scratch ------
// Callers that cannot allocate device memory (an external allocator owning
// the device, a fixed real-time budget) get this
// variant: its partial sums live in a fixed file-scope device array instead of
// a handle's buffer, so the entry point allocates nothing. The array is shared
// by every call; each call overwrites every partial it later reads, so nothing
// needs clearing, but overlapping calls race.
namespace {

constexpr long kNoAllocMaxChunks = 4096;
static_assert(GBG_NOALLOC_MAX_ENTRIES == kNoAllocMaxChunks * gbg::kLikChunk,
              "header limit and scratch size disagree");

static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxChunks * 3];

// Device address of g_noalloc_partials per CUDA context. A host-side name of
// a __device__ array is not a device address: the address is looked up with
// cudaGetSymbolAddress once per context, with that context current. Every
// context that loads the module has its own copy of the array (the primary
// context of each device, any context a caller created with the driver API,
// and the new primary context after cudaDeviceReset), so the cache is keyed
// by the driver's context ID, which the driver never reuses in a process.
// The two driver calls are resolved through the runtime, so the library keeps
// no link-time dependency on libcuda.
using CtxGetCurrentFn = int (*)(void **ctx);
using CtxGetIdFn = int (*)(void *ctx, unsigned long long *id);

struct NoAllocEntry {
    unsigned long long ctx_id;
    double *ptr;
};
constexpr int kMaxContexts = 64;
NoAllocEntry g_noalloc_cache[kMaxContexts];  // a ring: the oldest entry is replaced
int g_noalloc_count = 0, g_noalloc_next = 0;
std::mutex g_noalloc_mu;

int current_context_id(unsigned long long *id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        void *f1 = nullptr, *f2 = nullptr;
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        GBG_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1));
        GBG_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2));
        if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2) {
            gbg::set_error("gbg_loglik_noalloc: the driver lacks cuCtxGetCurrent/cuCtxGetId");
            return GBG_ERR_UNSUPPORTED;
        }
        get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    void *ctx = nullptr;
    if (get_current(&ctx) != 0 || !ctx || get_id(ctx, id) != 0) {
        gbg::set_error("gbg_loglik_noalloc: no current CUDA context");
        return GBG_ERR_CUDA;
    }
    return GBG_OK;
}

int noalloc_scratch(double **out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    unsigned long long id = 0;
    if (current_context_id(&id) != GBG_OK) {
        // no context bound to this thread yet: the runtime binds the current
        // device's primary context on its next call, then ask again
        int dev = -1;
        GBG_CUDA_TRY(cudaGetDevice(&dev));
        void *p = nullptr;
        GBG_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_partials));
        if (int rc = current_context_id(&id)) return rc;
    }
    for (int i = 0; i < g_noalloc_count; ++i)
        if (g_noalloc_cache[i].ctx_id == id) {
            *out = g_noalloc_cache[i].ptr;
            return GBG_OK;
        }
    void *p = nullptr;
    GBG_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_partials));
    g_noalloc_cache[g_noalloc_next] = {id, static_cast<double *>(p)};
    g_noalloc_next = (g_noalloc_next + 1) % kMaxContexts;
    if (g_noalloc_count < kMaxContexts) ++g_noalloc_count;
    *out = static_cast<double *>(p);
    return GBG_OK;
}

}  // namespace

extern "C" int gbg_loglik_noalloc(const float *phi_device, int n, const int *pet_idx,
                                  const double *pet_val, long n_pet, const int *ti_idx,
                                  const double *t1_val, const double *t2_val, long n_ti,
                                  const gbg_lik_params *p, gbg_lik_result *out_device,
                                  void *stream) {
    using namespace gbg;
    if (!phi_device || !p || !out_device || n < 1 || n_pet < 0 || n_ti < 0 ||
        (n_pet > 0 && (!pet_idx || !pet_val)) || (n_ti > 0 && (!ti_idx || !t1_val || !t2_val))) {
        set_error("gbg_loglik_noalloc: bad argument");
        return GBG_ERR_ARG;
    }
    if (n_pet > GBG_NOALLOC_MAX_ENTRIES || n_ti > GBG_NOALLOC_MAX_ENTRIES) {
        set_error("gbg_loglik_noalloc: list longer than GBG_NOALLOC_MAX_ENTRIES");
        return GBG_ERR_ARG;
    }
    if (!(p->pet_sigma2 > 0) || !(p->slope > 0)) {
        set_error("gbg_loglik_noalloc: likelihood parameters out of range");
        return GBG_ERR_ARG;
    }
    double *scratch = nullptr;
    if (int rc = noalloc_scratch(&scratch)) return rc;
    const long items = n_pet > n_ti ? n_pet : n_ti;
    const int chunks = items > 0 ? (int)((items + kLikChunk - 1) / kLikChunk) : 1;
    LikArgs a;
    a.n_pet = (int)n_pet;
    a.n_ti = (int)n_ti;
    a.chunks = chunks;
    a.pet_idx = pet_idx;
    a.pet_val = pet_val;
    a.ti_idx = ti_idx;
    a.t1_val = t1_val;
    a.t2_val = t2_val;
    a.pet_scale = p->pet_scale;
    a.t1_uc = p->t1_uc;
    a.t2_uc = p->t2_uc;
    a.is2 = 1. / p->slope;
    a.stride = (size_t)n * n * n;
    a.partials = scratch;
    PhiSource src{phi_device, phi_device, nullptr, nullptr};
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_lik_partial<<<dim3(chunks, 1), kLikThreads, 0, st>>>(a, src);
    k_lik_final<<<1, 128, 0, st>>>(scratch, chunks, 1, (int)n_pet, p->pet_sigma2, out_device);
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
}
