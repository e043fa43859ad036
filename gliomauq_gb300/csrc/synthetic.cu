// Synthetic observations from a tumour density, as the reference's
// synthetic-data program makes them (source/Glioma/Glioma_ProcessSyntheticData.cpp)
// in its default Real = float:
//   _ic (:61-104)             PET = u where u >= ucT2 else 0, T1 = [u >= ucT1],
//                             T2 = [u >= ucT2]   (u = the density as float)
//   run (:406-430)            statistics, normalise, noise, statistics,
//                             normalise
//   _getPETstatistic (:107-153)   max, and the centre of mass summed in float
//                             over the grid's loops in their order
//   _normalizePETsignal (:156-173) PET *= 1 / max (double)
//   _addNoise (:176-221)      drand48 pairs through Box-Muller: at every cell
//                             visited while the count of noised cells is
//                             even a new pair is drawn; a cell with PET > 0
//                             gets PET = max(0, PET + alpha xi_1) and passes
//                             xi_2 on as the next xi_1.
// The grid's loops visit the blocks in a given order (the reference's comes
// from MRAG's node map, ordered by node address), each block's cells with x
// fastest; that order decides which cell receives which random number and
// the float rounding of the sums, so it is an input here.
//
// On the GPU: the cells in loop order are indexed by an exclusive scan of
// the PET > 0 flags (the noised cells in order); the random numbers of the
// k-th noised cell follow from a scan over the gaps between noised cells
// (every cell in a gap before an even-numbered noised cell draws a pair) and
// a jump-ahead of drand48's linear congruential generator; the noise is then
// one thread per noised cell. The two statistics passes add in the loop
// order, as the reference does, on one thread over the noised cells only
// (the other cells add zeros). Compiled with -fmad=false.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "gbg_internal.cuh"

namespace gbg {
namespace {

constexpr int kScanTile = 1024;  // elements per block of the scan (256 threads x 4)
constexpr unsigned long long kLcgA = 0x5DEECE66Dull, kLcgC = 0xBull, kM48 = (1ull << 48) - 1;

// exclusive (or inclusive) scan of M ints, tile by tile; tile sums in `sums`
__global__ void k_scan_tiles(const int *__restrict__ in, int *__restrict__ out, long M, int inclusive,
                             int *__restrict__ sums) {
    __shared__ int s[kScanTile];
    const long base = (long)blockIdx.x * kScanTile;
    for (int i = threadIdx.x; i < kScanTile; i += blockDim.x) s[i] = base + i < M ? in[base + i] : 0;
    __syncthreads();
    // Hillis-Steele on the tile (inclusive)
    for (int off = 1; off < kScanTile; off <<= 1) {
        int v[4];
        for (int q = 0; q < 4; ++q) {
            const int i = threadIdx.x + q * blockDim.x;
            v[q] = i >= off ? s[i - off] : 0;
        }
        __syncthreads();
        for (int q = 0; q < 4; ++q) s[threadIdx.x + q * blockDim.x] += v[q];
        __syncthreads();
    }
    for (int i = threadIdx.x; i < kScanTile; i += blockDim.x)
        if (base + i < M) out[base + i] = inclusive ? s[i] : s[i] - (base + i < M ? in[base + i] : 0);
    if (threadIdx.x == 0) sums[blockIdx.x] = s[kScanTile - 1];
}

// exclusive scan of the tile sums on one block (tiles <= a few thousand)
__global__ void k_scan_sums(int *__restrict__ sums, int tiles, int *__restrict__ total) {
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int t = 0; t < tiles; ++t) {
            const int v = sums[t];
            sums[t] = acc;
            acc += v;
        }
        *total = acc;
    }
}

__global__ void k_scan_add(int *__restrict__ out, long M, const int *__restrict__ sums) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < M) out[i] += sums[i / kScanTile];
}

int scan_ints(cudaStream_t st, const int *in, int *out, long M, bool inclusive, int *sums, int *total) {
    const int tiles = (int)((M + kScanTile - 1) / kScanTile);
    k_scan_tiles<<<tiles, 256, 0, st>>>(in, out, M, inclusive ? 1 : 0, sums);
    k_scan_sums<<<1, 32, 0, st>>>(sums, tiles, total);
    k_scan_add<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(out, M, sums);
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
}

__global__ void k_syn_init(long N, const double *__restrict__ tumor, float uc1, float uc2, float *__restrict__ phi,
                           float *__restrict__ t1, float *__restrict__ t2) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N; c += (long)gridDim.x * blockDim.x) {
        const float u = (float)tumor[c];
        phi[c] = u >= uc2 ? u : 0.f;
        t1[c] = u >= uc1 ? 1.f : 0.f;
        t2[c] = u >= uc2 ? 1.f : 0.f;
    }
}

// trav[p] = the cell visited at loop position p; flag[p] = PET there > 0
__global__ void k_syn_order(long M, int n, const int4 *__restrict__ order, const float *__restrict__ phi,
                            int *__restrict__ trav, int *__restrict__ flag) {
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < M; p += (long)gridDim.x * blockDim.x) {
        const int4 b = order[p / 4096];
        const int l = (int)(p % 4096), x = l % 16, y = (l / 16) % 16, z = l / 256;
        const long c = (long)(16 * b.y + x) + (long)n * ((long)(16 * b.z + y) + (long)n * (16 * b.w + z));
        trav[p] = (int)c;
        flag[p] = phi[c] > 0.f ? 1 : 0;
    }
}

// list[k] = loop position of the k-th noised cell
__global__ void k_syn_compact(long M, const int *__restrict__ flag, const int *__restrict__ pos,
                              int *__restrict__ list) {
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < M; p += (long)gridDim.x * blockDim.x)
        if (flag[p]) list[pos[p]] = (int)p;
}

struct SynStats {
    float max, mass, c[3];
};

// _getPETstatistic over the noised cells in loop order (one thread)
__global__ void k_syn_stats(int K, const int *__restrict__ list, const int *__restrict__ trav,
                            const float *__restrict__ phi, int n, int level, SynStats *__restrict__ out) {
    if (threadIdx.x || blockIdx.x) return;
    const float hf = (float)(ldexp(1.0, -level) / 16.0);
    float mx = 0.f, mass = 0.f, cs[3] = {0.f, 0.f, 0.f};
    for (int k = 0; k < K; ++k) {
        const int c = trav[list[k]];
        const float p = phi[c];
        mx = mx < p ? p : mx;
        mass = __fadd_rn(mass, p);
        const int g[3] = {c % n, (c / n) % n, c / (n * n)};
        for (int j = 0; j < 3; ++j) {
            // BlockInfo::pos: origin + h * i, in float
            const float origin = (float)ldexp((double)(g[j] / 16), -level);
            const float x = __fadd_rn(origin, __fmul_rn(hf, (float)(g[j] % 16)));
            cs[j] = (float)__dadd_rn((double)cs[j], __dmul_rn((double)x, (double)p));
        }
    }
    out->max = mx;
    out->mass = mass;
    for (int j = 0; j < 3; ++j) out->c[j] = __fdiv_rn(cs[j], mass);
}

__global__ void k_syn_normalize(long N, float *__restrict__ phi, const SynStats *__restrict__ st) {
    const double iscale = 1.0 / (double)st->max;
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N; c += (long)gridDim.x * blockDim.x)
        phi[c] = (float)__dmul_rn((double)phi[c], iscale);
}

// g[k] = cells from the previous noised cell (exclusive) to the k-th
// (inclusive) when k is even: each of them draws a pair; 0 for odd k
__global__ void k_syn_gaps(int K, const int *__restrict__ list, int *__restrict__ g) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x)
        g[k] = (k & 1) ? 0 : list[k] - (k ? list[k - 1] : -1);
}

// drand48's state after `steps` draws from x0: the affine map x -> a x + c
// composed steps times, by squaring (everything mod 2^48; uint64 products
// are exact mod 2^64, hence mod 2^48)
__device__ unsigned long long lcg_jump(unsigned long long x0, unsigned long long steps) {
    unsigned long long A = 1, C = 0, a = kLcgA, c = kLcgC;
    while (steps) {
        if (steps & 1) {
            A = (A * a) & kM48;
            C = (C * a + c) & kM48;
        }
        c = (c * (a + 1)) & kM48;
        a = (a * a) & kM48;
        steps >>= 1;
    }
    return (A * x0 + C) & kM48;
}

__global__ void k_syn_noise(int K, const int *__restrict__ list, const int *__restrict__ trav,
                            const int *__restrict__ drawn, double alpha, unsigned long long seed,
                            float *__restrict__ phi) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x) {
        const unsigned long long m = (unsigned long long)drawn[k] - 1;  // the pair this cell uses
        const unsigned long long x1 = lcg_jump(seed, 2 * m + 1);
        const unsigned long long x2 = (kLcgA * x1 + kLcgC) & kM48;
        const double u1 = (double)x1 * (1.0 / 281474976710656.0), u2 = (double)x2 * (1.0 / 281474976710656.0);
        const double r = sqrt(-2.0 * log(u1));
        const double ang = (2.0 * 3.14159265358979323846) * u2;
        const double xi = (k & 1) ? r * sin(ang) : r * cos(ang);
        const int c = trav[list[k]];
        const double v = (double)phi[c] + alpha * xi;
        phi[c] = (float)(0.0 < v ? v : 0.0);
    }
}

__global__ void k_syn_out(long N, const float *__restrict__ phi, const float *__restrict__ t1,
                          const float *__restrict__ t2, double *__restrict__ o_pet, double *__restrict__ o_t1,
                          double *__restrict__ o_t2) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N; c += (long)gridDim.x * blockDim.x) {
        o_pet[c] = (double)phi[c];
        o_t1[c] = (double)t1[c];
        o_t2[c] = (double)t2[c];
    }
}

}  // namespace
}  // namespace gbg

extern "C" int gbg_synthetic_observations(int n, const double *tumor, int nblocks, const gbg_block *order,
                                          const gbg_synthetic_opts *o, double *pet, double *t1, double *t2,
                                          float *centre_of_mass) {
    using namespace gbg;
    int level = -1;
    for (int l = 0; l <= 8; ++l)
        if (n == (16 << l)) level = l;
    if (level < 0 || !tumor || !o || !pet || !t1 || !t2 || !centre_of_mass) {
        set_error("gbg_synthetic_observations: n must be 16 * 2^l (l <= 8) and every pointer set");
        return GBG_ERR_ARG;
    }
    const int side = 1 << level, nb = side * side * side;
    if (!(o->alpha >= 0) || !std::isfinite(o->alpha) || !std::isfinite(o->uc_t1) || !std::isfinite(o->uc_t2)) {
        set_error("gbg_synthetic_observations: bad thresholds or noise level");
        return GBG_ERR_ARG;
    }
    // the loop order: given, or blocks with x fastest
    std::vector<int4> ord(nb);
    if (order) {
        if (nblocks != nb) {
            set_error("gbg_synthetic_observations: the block order must list every block of the uniform grid");
            return GBG_ERR_ARG;
        }
        std::vector<char> seen(nb, 0);
        for (int b = 0; b < nb; ++b) {
            const gbg_block &g = order[b];
            if (g.level != level || g.ix < 0 || g.iy < 0 || g.iz < 0 || g.ix >= side || g.iy >= side ||
                g.iz >= side || seen[g.ix + side * (g.iy + side * g.iz)]++) {
                set_error("gbg_synthetic_observations: the block order is not a permutation of the grid's blocks");
                return GBG_ERR_ARG;
            }
            ord[b] = make_int4(g.level, g.ix, g.iy, g.iz);
        }
    } else {
        for (int b = 0; b < nb; ++b) ord[b] = make_int4(level, b % side, (b / side) % side, b / (side * side));
    }
    for (size_t i = 0, N = (size_t)n * n * n; i < N; ++i)
        if (!std::isfinite(tumor[i])) {
            set_error("gbg_synthetic_observations: non-finite density");
            return GBG_ERR_NONFINITE;
        }
    const long N = (long)n * n * n;
    const int tiles = (int)((N + kScanTile - 1) / kScanTile);
    int dev = 0, sms = 0;
    GBG_CUDA_TRY(cudaGetDevice(&dev));
    GBG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const unsigned grid = (unsigned)std::min<long>((N + 255) / 256, (long)sms * 8);
    // device working set
    const size_t bytes = N * (3 * sizeof(double) + 3 * sizeof(float) + 5 * sizeof(int)) + nb * sizeof(int4) +
                         (tiles + 2) * sizeof(int) + sizeof(SynStats) + 1024;
    char *w = nullptr;
    GBG_CUDA_TRY(cudaMalloc((void **)&w, bytes));
    char *q = w;
    auto carve = [&](size_t sz) {
        char *p = q;
        q += (sz + 255) & ~(size_t)255;
        return p;
    };
    double *d_io = (double *)carve(3 * N * sizeof(double));  // tumour in, then PET, T1, T2 out
    float *phi = (float *)carve(N * sizeof(float)), *ft1 = (float *)carve(N * sizeof(float)),
          *ft2 = (float *)carve(N * sizeof(float));
    int *trav = (int *)carve(N * sizeof(int)), *flag = (int *)carve(N * sizeof(int)),
        *pos = (int *)carve(N * sizeof(int)), *list = (int *)carve(N * sizeof(int)),
        *gap = (int *)carve(N * sizeof(int));
    int4 *d_ord = (int4 *)carve(nb * sizeof(int4));
    int *sums = (int *)carve((tiles + 2) * sizeof(int));
    int *total = sums + tiles;
    SynStats *st = (SynStats *)carve(sizeof(SynStats));
    cudaStream_t s = 0;
    int rc = GBG_OK;
    int K = 0;
    SynStats hs;
#define SYN_TRY(expr)                                                  \
    do {                                                               \
        cudaError_t _e = (expr);                                       \
        if (_e != cudaSuccess) {                                       \
            set_error(std::string(#expr) + ": " + cudaGetErrorString(_e)); \
            rc = GBG_ERR_CUDA;                                         \
            goto done;                                                 \
        }                                                              \
    } while (0)
    SYN_TRY(cudaMemcpyAsync(d_io, tumor, N * sizeof(double), cudaMemcpyHostToDevice, s));
    SYN_TRY(cudaMemcpyAsync(d_ord, ord.data(), nb * sizeof(int4), cudaMemcpyHostToDevice, s));
    k_syn_init<<<grid, 256, 0, s>>>(N, d_io, (float)o->uc_t1, (float)o->uc_t2, phi, ft1, ft2);
    k_syn_order<<<grid, 256, 0, s>>>(N, n, d_ord, phi, trav, flag);
    if ((rc = scan_ints(s, flag, pos, N, false, sums, total))) goto done;
    k_syn_compact<<<grid, 256, 0, s>>>(N, flag, pos, list);
    SYN_TRY(cudaGetLastError());
    SYN_TRY(cudaMemcpyAsync(&K, total, sizeof(int), cudaMemcpyDeviceToHost, s));
    SYN_TRY(cudaStreamSynchronize(s));
    if (K == 0) {
        set_error("gbg_synthetic_observations: no cell reaches the T2 threshold (the reference divides by 0)");
        rc = GBG_ERR_ARG;
        goto done;
    }
    // statistics, normalisation, noise, statistics, normalisation (run, :406-430)
    k_syn_stats<<<1, 32, 0, s>>>(K, list, trav, phi, n, level, st);
    k_syn_normalize<<<grid, 256, 0, s>>>(N, phi, st);
    if (o->alpha > 0) {
        const unsigned gk = (unsigned)std::min<long>((K + 255) / 256, (long)sms * 8);
        k_syn_gaps<<<gk, 256, 0, s>>>(K, list, gap);
        if ((rc = scan_ints(s, gap, flag, K, true, sums, total))) goto done;
        k_syn_noise<<<gk, 256, 0, s>>>(K, list, trav, flag, o->alpha, o->seed48 & kM48, phi);
    }
    k_syn_stats<<<1, 32, 0, s>>>(K, list, trav, phi, n, level, st);
    k_syn_normalize<<<grid, 256, 0, s>>>(N, phi, st);
    k_syn_out<<<grid, 256, 0, s>>>(N, phi, ft1, ft2, d_io, d_io + N, d_io + 2 * N);
    SYN_TRY(cudaGetLastError());
    SYN_TRY(cudaMemcpyAsync(pet, d_io, N * sizeof(double), cudaMemcpyDeviceToHost, s));
    SYN_TRY(cudaMemcpyAsync(t1, d_io + N, N * sizeof(double), cudaMemcpyDeviceToHost, s));
    SYN_TRY(cudaMemcpyAsync(t2, d_io + 2 * N, N * sizeof(double), cudaMemcpyDeviceToHost, s));
    SYN_TRY(cudaMemcpyAsync(&hs, st, sizeof(SynStats), cudaMemcpyDeviceToHost, s));
    SYN_TRY(cudaStreamSynchronize(s));
    for (int j = 0; j < 3; ++j) centre_of_mass[j] = hs.c[j];
done:
#undef SYN_TRY
    cudaFree(w);
    return rc;
}
