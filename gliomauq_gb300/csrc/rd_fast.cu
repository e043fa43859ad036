// Fast FP32 path and the batched population solver.
//
// Arithmetic (float storage, float math, FMA allowed):
//   k_c   = (p_w + r p_g) / (p_w + p_g)          unit diffusivity, r = Dg/Dw
//   c_f   = 2 k_c k_n / (k_c + k_n)              face coefficient (harmonic mean),
//                                                 precomputed per face in double
//   phi' = phi + a * sum_f c_f (phi_f - phi) + b * phi (1 - phi)
//          with a = dt * Dw / h^2 and b = dt * rho, clamped to [0, 1]
//   cells that are not tissue, or that touch a non-tissue face neighbour,
//   are set to 0 (mask = 0)
// This is the reference's Case2 operator (source/Glioma/Glioma_ReactionDiffusionOperator.h:174-216)
// written with Dw factored out of the face diffusivities, the flux sum written
// as sum c_f (phi_f - phi), and its boundary behaviour stated as a mask: in
// the reference a tissue cell with a face neighbour of zero tissue fraction
// gets df = 0/0 = NaN, hence phi = max(0, NaN) = 0 every step, and a
// non-tissue cell stays at 0.
//
// Data layout in HBM: one n^3 float field per sample, x fastest, samples
// contiguous (sample s at s*n^3); coefficient fields cx, cy, cz (face to the
// +x/+y/+z neighbour) and the mask as four n^3 float arrays shared by every
// sample.
//
// Thread mapping: a warp segment of n/4 lanes covers one x-row, each lane
// four consecutive cells (float4); x-neighbours across lanes come by shuffle
// within the segment, which also wraps the periodic x boundary. A 256-thread
// CTA covers 256/(n/4) rows in y and marches TZ planes in z, keeping the
// z-1, z, z+1 planes of its cells in registers.
//
// The density buffers are rewritten inside one launch (they alternate between
// input and output every round), so they are read with __ldcg (L2, coherent)
// and never through the read-only path; the anatomy tables use __ldg.
//
// Population schedule: a persistent cooperative kernel advances every active
// sample by one step per round, rounds separated by a bounded grid barrier.
// Samples are ordered by step count, longest first, so the active samples of
// round k are a prefix of that order.
//
// Kernel families (the autotuner times them per grid size): the skipping
// kernel (k_population10, the batched solver's default: k_population8's tile
// march over only the tiles whose output can be nonzero -- tiles with a live
// cell, inside each sample's initial support grown by a cell per step);
// registers (k_population8: planes carried in registers, the mask in the sign
// bit of the x-face table, 32-bit offsets; k_population9: the same with two
// samples of one tile per warp sharing the anatomy loads); a bulk-copy ring
// fed by the TMA unit with mbarrier completion and a producer warp
// (k_population6); and temporal blocking (k_population7: two steps per round
// through a shared-memory ring of first-step planes, density read and written
// once per two steps). All run the same per-cell operation sequence, so every
// variant gives the same bits.
#include <cstdio>
#include <vector>

#include "gbg_internal.cuh"

namespace gbg {

namespace {

__device__ __forceinline__ int wrapm(int i, int n) { return i == 0 ? n - 1 : i - 1; }
__device__ __forceinline__ int wrapp(int i, int n) { return i == n - 1 ? 0 : i + 1; }

__global__ void k_fast_tables(int n, const double *__restrict__ pw, const double *__restrict__ pg,
                              double ratio, float *__restrict__ cx, float *__restrict__ cy,
                              float *__restrict__ cz, float *__restrict__ msk,
                              float *__restrict__ cxs) {
    const size_t N = (size_t)n * n * n;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
         c += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(c % n), y = (int)((c / n) % n), z = (int)(c / ((size_t)n * n));
        const size_t nn = n;
        const size_t nb[7] = {c,
                              c - x + wrapp(x, n),
                              c + ((size_t)wrapp(y, n) - y) * nn,
                              c + ((size_t)wrapp(z, n) - z) * nn * nn,
                              c - x + wrapm(x, n),
                              c + ((size_t)wrapm(y, n) - y) * nn,
                              c + ((size_t)wrapm(z, n) - z) * nn * nn};
        double k[4];
        bool all = true;
        for (int i = 0; i < 7; ++i) {
            const double b = pw[nb[i]] + pg[nb[i]];
            all = all && (b > 0.0);
            if (i < 4) k[i] = b > 0.0 ? (pw[nb[i]] + ratio * pg[nb[i]]) / b : 0.0;
        }
        float *dst[3] = {cx, cy, cz};
        for (int f = 0; f < 3; ++f) {
            const double s = k[0] + k[f + 1];
            dst[f][c] = (k[0] > 0.0 && k[f + 1] > 0.0 && s > 0.0) ? (float)(2.0 * k[0] * k[f + 1] / s) : 0.0f;
        }
        msk[c] = all ? 1.0f : 0.0f;
        // every coefficient is +0 or positive, so the sign bit is free to carry
        // the mask: |cxs| = cx exactly, signbit(cxs) = (msk == 0)
        cxs[c] = all ? cx[c] : -cx[c];
    }
}

// Reference time loop per sample (Glioma_HG_UQ.cpp:532-552): Dw /= L^2;
// Dg = 0.1 Dw; dt = 0.99 h^2 / (6 max(Dw, Dg)); steps while t <= tend.
// f32 rounds Dw and Dg to float as the default build does. Explicit _rn
// intrinsics keep every operation rounded on its own.
__global__ void k_schedule(const gbg_sample *__restrict__ smp, int S, int n, double L, int f32,
                           SampleRec *__restrict__ unsorted) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const double h = __ddiv_rn(1.0, (double)n);
    double Dw, Dg, rho;
    if (f32) {
        const float dwf = (float)__ddiv_rn((double)(float)smp[s].Dw, __dmul_rn(L, L));
        const float dgf = (float)__dmul_rn(0.1, (double)dwf);
        Dw = dwf;
        Dg = dgf;
        rho = (double)(float)smp[s].rho;
    } else {
        Dw = __ddiv_rn(smp[s].Dw, __dmul_rn(L, L));
        Dg = __dmul_rn(0.1, Dw);
        rho = smp[s].rho;
    }
    const double mx = Dw >= Dg ? Dw : Dg;
    const double dt = __ddiv_rn(__dmul_rn(__dmul_rn(0.99, h), h), __dmul_rn(__dmul_rn(2., 3.), mx));
    int k = 0;
    double t = 0.0;
    const double tend = smp[s].tend;
    // bounded: at most 10^8 steps per sample
    while (t <= tend && k < 100000000) {
        t = __dadd_rn(t, dt);
        ++k;
    }
    const double ih2 = __ddiv_rn(1., __dmul_rn(h, h));
    SampleRec r;
    r.a = (float)(dt * Dw * ih2);
    r.b = (float)(dt * rho);
    r.nsteps = k;
    r.order = s;
    r.dt = dt;
    r.a2 = r.a;
    r.b2 = r.b;
    unsorted[s] = r;
}

// Smooth time grids: a step dt, k = ceil(tend/dt) steps (at least one), the
// last of length tend - (k-1) dt, so the final state is continuous in tend.
//   dt0 > 0: dt = dt0 for every sample (fixed grid)
//   dt0 < 0: dt = |dt0| * 0.99 h^2 / (6 Dw / L^2 + rho h^2 / 2) per sample
//            (scaled grid): the reference's step rule with the reaction's
//            share of the stability bound added. The reference's rule alone
//            bounds only the diffusion part: where phi is near 1 the
//            checkerboard mode of a white-matter region then grows by
//            |1 - 12 a - b| > 1 per step, the clamp to [0, 1] bounds it, and
//            the final density amplifies rounding differences. Here
//            12 a + b = 1.98 |dt0| for every sample, so that mode decays. a =
//            dt Dw / h^2 and b = dt rho depend on rho h^2 L^2 / Dw only and
//            the step count on tend times a function of the same ratio: the
//            discrete model keeps the continuous one's symmetry
//            (Dw, rho, tend) -> (c Dw, c rho, tend / c).
// Dw in double (no float rounding of the input); every operation rounded on
// its own so host code that restates it gets the same coefficients.
// 6 Dw + rho h^2 / 2 (Dw in unit-cube units), rounded operation by operation
__device__ __forceinline__ double scaled_grid_den(double Dw, double rho, double h) {
    return __dadd_rn(__dmul_rn(6.0, Dw), __dmul_rn(__dmul_rn(0.5, rho), __dmul_rn(h, h)));
}

__global__ void k_schedule_smooth(const gbg_sample *__restrict__ smp, int S, int n, double L, double dt0,
                                  SampleRec *__restrict__ unsorted) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const double h = __ddiv_rn(1.0, (double)n);
    const double ih2 = __ddiv_rn(1., __dmul_rn(h, h));
    const double Dw = __ddiv_rn(smp[s].Dw, __dmul_rn(L, L));
    const double rho = smp[s].rho, tend = smp[s].tend;
    double dt = dt0;
    if (dt0 < 0)
        dt = __dmul_rn(-dt0, __ddiv_rn(__dmul_rn(__dmul_rn(0.99, h), h), scaled_grid_den(Dw, rho, h)));
    double kk = ceil(__ddiv_rn(tend, dt));
    if (!(kk >= 1.0)) kk = 1.0;
    if (kk > 1e8) kk = 1e8;
    const int k = (int)kk;
    const double dtl = __dadd_rn(tend, -__dmul_rn((double)(k - 1), dt));
    SampleRec r;
    r.a = (float)__dmul_rn(__dmul_rn(dt, Dw), ih2);
    r.b = (float)__dmul_rn(dt, rho);
    r.a2 = (float)__dmul_rn(__dmul_rn(dtl, Dw), ih2);
    r.b2 = (float)__dmul_rn(dtl, rho);
    r.nsteps = k;
    r.order = s;
    r.dt = dt;
    unsorted[s] = r;
}

// Stable rank by nsteps descending; S is small (<= a few thousand).
__global__ void k_sort_schedule(const SampleRec *__restrict__ unsorted, int S,
                                SampleRec *__restrict__ sorted, int *__restrict__ rank_of) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const int ks = unsorted[s].nsteps;
    int r = 0;
    for (int j = 0; j < S; ++j) {
        const int kj = unsorted[j].nsteps;
        r += (kj > ks) || (kj == ks && j < s);
    }
    sorted[r] = unsorted[s];
    rank_of[s] = r;
}

// phi1 and recs non-null (temporally blocked population kernels): sample s
// starts in phi1 when (nsteps_s / 2) is odd, so that its final state lands in
// buffer nsteps_s & 1 like every other population kernel's.
__device__ __forceinline__ float gaussian_ic_value(int x, int y, int z, double x0, double y0, double z0,
                                                   double peak, double two_s2, float screen,
                                                   const double *__restrict__ pw, const double *__restrict__ pg,
                                                   unsigned c) {
    // float screen: cells with d^2 > 2 sigma^2 * 120 (+1 voxel^2 margin for the
    // float rounding) have exponent < -110 and get 0 below; skip their FP64 work
    const float fx = (float)x - (float)x0, fy = (float)y - (float)y0, fz = (float)z - (float)z0;
    const bool near = peak > 1.0 || fx * fx + fy * fy + fz * fz <= screen;
    float v = 0.0f;
    if (near && pw[c] + pg[c] > 0.0) {
        // d2 and the exponent rounded operation by operation (no FMA), as
        // peak * exp(-d2 / (2 sigma^2)) evaluates in plain double arithmetic
        const double dx = x - x0, dy = y - y0, dz = z - z0;
        const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
        const double e = __ddiv_rn(-d2, two_s2);
        // below -745 exp underflows to 0; below -110 peak*exp(e) <= 1e-47
        // rounds to float 0 for any peak <= 1e+0: skip the FP64 exp there
        if (e > -110.0 || peak > 1.0) v = (float)__dmul_rn(peak, exp(e));
    }
    return v;
}

// Grid: y over samples, x over groups of four consecutive cells of one
// sample (float4 stores when n is a multiple of 4, cell by cell otherwise).
// 32-bit index arithmetic inside a sample (n <= 1024, n^3 < 2^32).
// box non-null (the skipping population kernel): the y and z extent of the
// cells given a nonzero value is recorded per sample as four ints
// {n - ymin, ymax + 1, n - zmin, zmax + 1} (all 0: no nonzero cell) with
// atomicMax, from zero-filled entries.
__device__ __forceinline__ void record_support(int *box, int n, int y, int z) {
    atomicMax(box + 0, n - y);
    atomicMax(box + 1, y + 1);
    atomicMax(box + 2, n - z);
    atomicMax(box + 3, z + 1);
}

__global__ void k_gaussian_ic(int n, const gbg_sample *__restrict__ smp, int S, double peak,
                              double sigma, const double *__restrict__ pw, const double *__restrict__ pg,
                              float *__restrict__ phi, float *__restrict__ phi1 = nullptr,
                              const SampleRec *__restrict__ recs = nullptr, int *__restrict__ box = nullptr) {
    const unsigned un = (unsigned)n, N = un * un * un, groups = (N + 3) / 4;
    const double two_s2 = __dmul_rn(__dmul_rn(2.0, sigma), sigma);
    const float screen = (float)(two_s2 * 120.0) + 1.0f;
    for (unsigned s = blockIdx.y; s < (unsigned)S; s += gridDim.y) {
        const double x0 = smp[s].x0, y0 = smp[s].y0, z0 = smp[s].z0;
        float *dst = ((phi1 && recs && ((recs[s].nsteps / 2) & 1)) ? phi1 : phi) + (size_t)s * N;
        for (unsigned g = blockIdx.x * blockDim.x + threadIdx.x; g < groups; g += gridDim.x * blockDim.x) {
            const unsigned c = 4 * g;
            if ((un & 3u) == 0) {
                const unsigned row = c / un;
                const int x = (int)(c - row * un), y = (int)(row % un), z = (int)(row / un);
                float v[4];
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    v[j] = gaussian_ic_value(x + j, y, z, x0, y0, z0, peak, two_s2, screen, pw, pg, c + j);
                *reinterpret_cast<float4 *>(dst + c) = make_float4(v[0], v[1], v[2], v[3]);
                if (box && (v[0] != 0.0f || v[1] != 0.0f || v[2] != 0.0f || v[3] != 0.0f))
                    record_support(box + 4 * s, n, y, z);
            } else {
                for (unsigned cj = c; cj < c + 4 && cj < N; ++cj) {
                    const unsigned row = cj / un;
                    const float v = gaussian_ic_value((int)(cj - row * un), (int)(row % un), (int)(row / un), x0,
                                                      y0, z0, peak, two_s2, screen, pw, pg, cj);
                    dst[cj] = v;
                    if (box && v != 0.0f) record_support(box + 4 * s, n, (int)(row % un), (int)(row / un));
                }
            }
        }
    }
}

dim3 ic_grid(const Handle &h, int S) {
    const unsigned groups = (unsigned)((h.N + 3) / 4);
    unsigned gx = (groups + 255) / 256;
    if (gx > 128) gx = 128;
    unsigned gy = (unsigned)h.num_sms * 16 / gx;
    if (gy < 1) gy = 1;
    if (gy > (unsigned)S) gy = (unsigned)S;
    if (gy > 65535) gy = 65535;
    return dim3(gx, gy);
}

// Bounded grid barrier for the cooperative persistent kernel. Returns false
// (and records DEV_BARRIER_TIMEOUT) if the other CTAs do not arrive within
// the spin limit; the caller then leaves the kernel.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, int *status, unsigned nblocks) {
    __syncthreads();
    __shared__ int ok;
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = bar + 1;
        const unsigned gen = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(bar, 1u);
        int good = 1;
        if (arrived == nblocks - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long spins = 0;
            while (*vgen == gen) {
                __nanosleep(64);
                if (++spins > (1ll << 25)) {  // ~ a few seconds
                    atomicExch(status, (int)DEV_BARRIER_TIMEOUT);
                    good = 0;
                    break;
                }
                if ((spins & 1023) == 0 && *(volatile int *)status != DEV_OK) {
                    good = 0;
                    break;
                }
            }
        }
        __threadfence();
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

struct PopArgs {
    int n, S, TZ, tiles_y, tiles;  // tiles per sample = tiles_y * (n / TZ)
    size_t stride;                 // cells per sample field
    float *buf0, *buf1;
    // k_population8<..., SLOT = true> only: every state kept, step k reading
    // buf0 + k * slot and writing buf0 + (k + 1) * slot (floats)
    size_t slot;
    const float *cx, *cy, *cz, *msk;
    const float *cxs;              // cx, sign bit = not msk
    const SampleRec *rec;          // sorted by nsteps descending
    unsigned *barrier;
    int *status;
    // skipping kernel only: live tiles, per-tile liveness, initial-support
    // boxes (unsorted sample order, see k_gaussian_ic)
    const int *live_list, *live_count;
    const unsigned char *tile_live;
    const int *box;
    int grow0;  // the first buffer's support lies within the boxes grown by grow0 cells
    unsigned long long *visited;  // tiles computed by this launch (k_population8/10)
};

// Register variant with fewer loads and cheaper addressing: the mask comes
// from the sign bit of the x-face table (one float4 load less per plane), and
// offsets inside a sample are 32-bit, formed once per tile and advanced by a
// plane per step. The mask is applied as the sign bit of cxs (|cxs| = cx).
template <int LR>
__device__ __forceinline__ void march_tile_s(int n, int TZ, int ty0, int tz0,
                                             const float *__restrict__ in, float *__restrict__ out,
                                             const float *__restrict__ cxs, const float *__restrict__ cy,
                                             const float *__restrict__ cz, float a, float b) {
    const int lane = threadIdx.x & 31;
    const int li = lane % LR;
    const int y = ty0 + (int)(threadIdx.x / LR);
    const int x0 = 4 * li;
    const int ym = wrapm(y, n), yp = wrapp(y, n);
    const unsigned plane = (unsigned)n * (unsigned)n;
    const unsigned oy = (unsigned)(x0 + n * y), oym = (unsigned)(x0 + n * ym), oyp = (unsigned)(x0 + n * yp);
    auto ld = [](const float *base, unsigned off) { return __ldcg(reinterpret_cast<const float4 *>(base + off)); };
    auto lg = [](const float *base, unsigned off) { return __ldg(reinterpret_cast<const float4 *>(base + off)); };
    const unsigned zso = plane * (unsigned)wrapm(tz0, n);
    unsigned zo = plane * (unsigned)tz0;
    float4 Pp = ld(in, oy + zso);
    float4 Pc = ld(in, oy + zo);
    float4 CZp = lg(cz, oy + zso);
    const unsigned last = plane * (unsigned)(n - 1);
    for (int dz = 0; dz < TZ; ++dz) {
        const unsigned zno = zo == last ? 0u : zo + plane;
        const float4 Pn = ld(in, oy + zno);
        const float4 PS = ld(in, oym + zo);
        const float4 PN = ld(in, oyp + zo);
        const float4 CX = lg(cxs, oy + zo);
        const float4 CY = lg(cy, oy + zo);
        const float4 CYm = lg(cy, oym + zo);
        const float4 CZ = lg(cz, oy + zo);
        const float left = __shfl_sync(0xffffffffu, Pc.w, (li + LR - 1) % LR, LR);
        const float right = __shfl_sync(0xffffffffu, Pc.x, (li + 1) % LR, LR);
        const float cxl = __shfl_sync(0xffffffffu, CX.w, (li + LR - 1) % LR, LR);
        const float p[6] = {left, Pc.x, Pc.y, Pc.z, Pc.w, right};
        const float cxa[5] = {fabsf(cxl), fabsf(CX.x), fabsf(CX.y), fabsf(CX.z), fabsf(CX.w)};
        const bool off4[4] = {signbit(CX.x), signbit(CX.y), signbit(CX.z), signbit(CX.w)};
        const float ps[4] = {PS.x, PS.y, PS.z, PS.w}, pn[4] = {PN.x, PN.y, PN.z, PN.w};
        const float pp[4] = {Pp.x, Pp.y, Pp.z, Pp.w}, pq[4] = {Pn.x, Pn.y, Pn.z, Pn.w};
        const float cy4[4] = {CY.x, CY.y, CY.z, CY.w}, cym4[4] = {CYm.x, CYm.y, CYm.z, CYm.w};
        const float cz4[4] = {CZ.x, CZ.y, CZ.z, CZ.w}, czp4[4] = {CZp.x, CZp.y, CZp.z, CZp.w};
        float o[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float f0 = p[i + 1];
            float lap = cxa[i] * (p[i] - f0);
            lap = fmaf(cxa[i + 1], p[i + 2] - f0, lap);
            lap = fmaf(cym4[i], ps[i] - f0, lap);
            lap = fmaf(cy4[i], pn[i] - f0, lap);
            lap = fmaf(czp4[i], pp[i] - f0, lap);
            lap = fmaf(cz4[i], pq[i] - f0, lap);
            float v = fmaf(a, lap, f0);
            v = fmaf(b * f0, 1.0f - f0, v);
            v = fminf(fmaxf(v, 0.0f), 1.0f);
            o[i] = off4[i] ? 0.0f : v;
        }
        *reinterpret_cast<float4 *>(out + oy + zo) = make_float4(o[0], o[1], o[2], o[3]);
        Pp = Pc;
        Pc = Pn;
        CZp = CZ;
        zo = zno;
    }
}

template <int LR, int MINB, bool SLOT = false>
__global__ void __launch_bounds__(256, MINB) k_population8(PopArgs p) {
    const int maxsteps = p.S > 0 ? p.rec[0].nsteps : 0;
    int active = p.S;
    const int rows = 256 / LR;
    unsigned long long visited = 0;
    for (int k = 0; k < maxsteps; ++k) {
        while (active > 0 && p.rec[active - 1].nsteps <= k) --active;
        const float *in = SLOT ? p.buf0 + (size_t)k * p.slot : ((k & 1) ? p.buf1 : p.buf0);
        float *out = SLOT ? p.buf0 + (size_t)(k + 1) * p.slot : ((k & 1) ? p.buf0 : p.buf1);
        const long items = (long)active * p.tiles;
        for (long it = blockIdx.x; it < items; it += gridDim.x) {
            const int r = (int)(it % active), t = (int)(it / active);
            const int ty = t % p.tiles_y, tz = t / p.tiles_y;
            const size_t off = (size_t)p.rec[r].order * p.stride;
            const bool last = k == p.rec[r].nsteps - 1;
            march_tile_s<LR>(p.n, p.TZ, ty * rows, tz * p.TZ, in + off, out + off, p.cxs, p.cy, p.cz,
                             last ? p.rec[r].a2 : p.rec[r].a, last ? p.rec[r].b2 : p.rec[r].b);
            ++visited;
        }
        if (k + 1 < maxsteps && !grid_barrier(p.barrier, p.status, gridDim.x)) break;
    }
    if (threadIdx.x == 0 && visited) atomicAdd(p.visited, visited);
}

// Skipping variant of k_population8: a round visits only the tiles whose
// output can be nonzero, with the same per-cell operation sequence, so the
// results are bitwise those of the dense kernels.
//   * A tile none of whose cells has mask 1 writes only zeros (masked cells
//     get 0 whatever their inputs).
//   * The output of round k can be nonzero only within one cell of the input's
//     support, so inside the initial support's y/z box grown by k + 1 cells (a
//     grown range reaching past a face covers the whole periodic axis); a
//     tile outside it writes only zeros too (with inputs that are all +0 the
//     step gives +0).
// A skipped tile therefore has to hold zeros in the output buffer already:
// the second buffer is zero-filled before the launch, the first holds the
// initial state, which is zero outside the initial support. Round 0 reads the
// initial state, which can be nonzero on masked tissue cells next to the
// non-tissue region; round 1 writes that buffer, so it also rewrites (with
// zeros) every tile without a live cell that meets the initial support. A
// live tile, once visited, is visited in every later round of its sample (the
// boxes only grow), so from round 2 on both buffers hold zeros in every tile a
// round skips.
__device__ __forceinline__ bool span_hits(int lo, int hi, int grow, int a, int b, int n) {
    lo -= grow;
    hi += grow;
    if (lo < 0 || hi > n - 1) return true;
    return lo <= b && a <= hi;
}

// Zeros over a tile of rows x TZ planes (march_tile_s's thread mapping).
template <int LR>
__device__ __forceinline__ void zero_tile(int n, int TZ, int ty0, int tz0, float *__restrict__ out) {
    const int x0 = 4 * ((threadIdx.x & 31) % LR);
    const int y = ty0 + (int)(threadIdx.x / LR);
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int z = tz0; z < tz0 + TZ; ++z)
        *reinterpret_cast<float4 *>(out + x0 + (size_t)n * ((size_t)y + (size_t)n * z)) = z4;
}

// SLOT = true keeps every state (step k reads buf0 + k * slot, writes
// buf0 + (k + 1) * slot): every round visits every tile of its active
// samples, computing those the rule above keeps and writing zeros over the
// others (a slot's previous contents are arbitrary), so each state is
// complete.
template <int LR, int MINB, bool SLOT = false>
__global__ void __launch_bounds__(256, MINB) k_population10(PopArgs p) {
    const int maxsteps = p.S > 0 ? p.rec[0].nsteps : 0;
    int active = p.S;
    const int rows = 256 / LR;
    const int n = p.n;
    const int nlive = SLOT ? p.tiles : *p.live_count;
    unsigned long long visited = 0;
    for (int k = 0; k < maxsteps; ++k) {
        while (active > 0 && p.rec[active - 1].nsteps <= k) --active;
        const float *in = SLOT ? p.buf0 + (size_t)k * p.slot : ((k & 1) ? p.buf1 : p.buf0);
        float *out = SLOT ? p.buf0 + (size_t)(k + 1) * p.slot : ((k & 1) ? p.buf0 : p.buf1);
        const int ntiles = (SLOT || k == 1) ? p.tiles : nlive;
        const long items = (long)active * ntiles;
        for (long it = blockIdx.x; it < items; it += gridDim.x) {
            const int r = (int)(it % active), ti = (int)(it / active);
            const int t = (SLOT || k == 1) ? ti : p.live_list[ti];
            const int order = p.rec[r].order;
            const size_t off = (size_t)order * p.stride;
            const int4 bx = reinterpret_cast<const int4 *>(p.box)[order];
            const int y0 = (t % p.tiles_y) * rows, z0 = (t / p.tiles_y) * p.TZ;
            if (bx.y == 0) {  // no nonzero initial cell: the sample stays 0
                if (SLOT) zero_tile<LR>(n, p.TZ, y0, z0, out + off);
                continue;
            }
            const int ylo = n - bx.x, yhi = bx.y - 1, zlo = n - bx.z, zhi = bx.w - 1;
            const int y1 = y0 + rows - 1, z1 = z0 + p.TZ - 1;
            const int g = p.grow0 + k + 1;
            bool go = span_hits(ylo, yhi, g, y0, y1, n) && span_hits(zlo, zhi, g, z0, z1, n);
            if (SLOT)
                go = go && p.tile_live[t];
            else if (go && k == 1 && !p.tile_live[t])
                go = span_hits(ylo, yhi, p.grow0, y0, y1, n) && span_hits(zlo, zhi, p.grow0, z0, z1, n);
            if (!go) {
                if (SLOT) zero_tile<LR>(n, p.TZ, y0, z0, out + off);
                continue;
            }
            const bool last = k == p.rec[r].nsteps - 1;
            march_tile_s<LR>(n, p.TZ, y0, z0, in + off, out + off, p.cxs, p.cy, p.cz,
                             last ? p.rec[r].a2 : p.rec[r].a, last ? p.rec[r].b2 : p.rec[r].b);
            ++visited;
        }
        if (k + 1 < maxsteps && !grid_barrier(p.barrier, p.status, gridDim.x)) break;
    }
    if (threadIdx.x == 0 && visited) atomicAdd(p.visited, visited);
}

// Liveness of the tiles of rows x tz cells (full x-rows): one CTA per tile,
// a tile is live when a cell has the mask (sign bit of cxs clear).
__global__ void k_tile_live(int n, int rows, int tz, const float *__restrict__ cxs, unsigned char *__restrict__ live) {
    const int tiles_y = n / rows;
    const int t = blockIdx.x;
    const int y0 = (t % tiles_y) * rows, z0 = (t / tiles_y) * tz;
    const unsigned cells = (unsigned)rows * (unsigned)tz * (unsigned)n;
    int any = 0;
    for (unsigned i = threadIdx.x; i < cells; i += blockDim.x) {
        const unsigned x = i % (unsigned)n, yz = i / (unsigned)n;
        const unsigned y = (unsigned)y0 + yz % (unsigned)rows, z = (unsigned)z0 + yz / (unsigned)rows;
        any |= !signbit(cxs[x + (size_t)n * (y + (size_t)n * z)]);
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) live[t] = (unsigned char)(any != 0);
}

// Live tile indices in increasing order (one thread: at most a few thousand tiles).
__global__ void k_compact_live(int tiles, const unsigned char *__restrict__ live, int *__restrict__ list,
                               int *__restrict__ count) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int c = 0;
    for (int t = 0; t < tiles; ++t)
        if (live[t]) list[c++] = t;
    *count = c;
}

// Two samples on one tile per warp: the anatomy (cxs, cy, cz) is loaded once
// for both, so a plane costs 6 density + 4 anatomy loads for two samples
// (5 per sample in place of 7), and each round trip of loads feeds twice the
// arithmetic. The second slot is idle (two = false) for the odd sample of a
// round. Per-sample operation sequence as march_tile_s.
template <int LR>
__device__ __forceinline__ void stencil4(const float4 &Pc, const float4 &Pp, const float4 &Pn, const float4 &PS,
                                         const float4 &PN, const float4 &CX, const float4 &CY,
                                         const float4 &CYm, const float4 &CZ, const float4 &CZp, float cxl,
                                         int li, float a, float b, float4 &res) {
    const float left = __shfl_sync(0xffffffffu, Pc.w, (li + LR - 1) % LR, LR);
    const float right = __shfl_sync(0xffffffffu, Pc.x, (li + 1) % LR, LR);
    const float p[6] = {left, Pc.x, Pc.y, Pc.z, Pc.w, right};
    const float cxa[5] = {fabsf(cxl), fabsf(CX.x), fabsf(CX.y), fabsf(CX.z), fabsf(CX.w)};
    const bool off4[4] = {signbit(CX.x), signbit(CX.y), signbit(CX.z), signbit(CX.w)};
    const float ps[4] = {PS.x, PS.y, PS.z, PS.w}, pn[4] = {PN.x, PN.y, PN.z, PN.w};
    const float pp[4] = {Pp.x, Pp.y, Pp.z, Pp.w}, pq[4] = {Pn.x, Pn.y, Pn.z, Pn.w};
    const float cy4[4] = {CY.x, CY.y, CY.z, CY.w}, cym4[4] = {CYm.x, CYm.y, CYm.z, CYm.w};
    const float cz4[4] = {CZ.x, CZ.y, CZ.z, CZ.w}, czp4[4] = {CZp.x, CZp.y, CZp.z, CZp.w};
    float o[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float f0 = p[i + 1];
        float lap = cxa[i] * (p[i] - f0);
        lap = fmaf(cxa[i + 1], p[i + 2] - f0, lap);
        lap = fmaf(cym4[i], ps[i] - f0, lap);
        lap = fmaf(cy4[i], pn[i] - f0, lap);
        lap = fmaf(czp4[i], pp[i] - f0, lap);
        lap = fmaf(cz4[i], pq[i] - f0, lap);
        float v = fmaf(a, lap, f0);
        v = fmaf(b * f0, 1.0f - f0, v);
        v = fminf(fmaxf(v, 0.0f), 1.0f);
        o[i] = off4[i] ? 0.0f : v;
    }
    res = make_float4(o[0], o[1], o[2], o[3]);
}

template <int LR>
__device__ __forceinline__ void march_tile_pair(int n, int TZ, int ty0, int tz0, bool two,
                                                const float *__restrict__ in0, float *__restrict__ out0,
                                                const float *__restrict__ in1, float *__restrict__ out1,
                                                const float *__restrict__ cxs, const float *__restrict__ cy,
                                                const float *__restrict__ cz, float a0, float b0, float a1,
                                                float b1) {
    const int lane = threadIdx.x & 31;
    const int li = lane % LR;
    const int y = ty0 + (int)(threadIdx.x / LR);
    const int x0 = 4 * li;
    const int ym = wrapm(y, n), yp = wrapp(y, n);
    const unsigned plane = (unsigned)n * (unsigned)n;
    const unsigned oy = (unsigned)(x0 + n * y), oym = (unsigned)(x0 + n * ym), oyp = (unsigned)(x0 + n * yp);
    auto ld = [](const float *base, unsigned off) { return __ldcg(reinterpret_cast<const float4 *>(base + off)); };
    auto lg = [](const float *base, unsigned off) { return __ldg(reinterpret_cast<const float4 *>(base + off)); };
    const unsigned zso = plane * (unsigned)wrapm(tz0, n);
    unsigned zo = plane * (unsigned)tz0;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 Pp0 = ld(in0, oy + zso), Pc0 = ld(in0, oy + zo);
    float4 Pp1 = two ? ld(in1, oy + zso) : zero, Pc1 = two ? ld(in1, oy + zo) : zero;
    float4 CZp = lg(cz, oy + zso);
    const unsigned last = plane * (unsigned)(n - 1);
    for (int dz = 0; dz < TZ; ++dz) {
        const unsigned zno = zo == last ? 0u : zo + plane;
        const float4 Pn0 = ld(in0, oy + zno), PS0 = ld(in0, oym + zo), PN0 = ld(in0, oyp + zo);
        float4 Pn1 = zero, PS1 = zero, PN1 = zero;
        if (two) {
            Pn1 = ld(in1, oy + zno);
            PS1 = ld(in1, oym + zo);
            PN1 = ld(in1, oyp + zo);
        }
        const float4 CX = lg(cxs, oy + zo);
        const float4 CY = lg(cy, oy + zo);
        const float4 CYm = lg(cy, oym + zo);
        const float4 CZ = lg(cz, oy + zo);
        const float cxl = __shfl_sync(0xffffffffu, CX.w, (li + LR - 1) % LR, LR);
        float4 r0, r1;
        stencil4<LR>(Pc0, Pp0, Pn0, PS0, PN0, CX, CY, CYm, CZ, CZp, cxl, li, a0, b0, r0);
        *reinterpret_cast<float4 *>(out0 + oy + zo) = r0;
        if (two) {
            stencil4<LR>(Pc1, Pp1, Pn1, PS1, PN1, CX, CY, CYm, CZ, CZp, cxl, li, a1, b1, r1);
            *reinterpret_cast<float4 *>(out1 + oy + zo) = r1;
        }
        Pp0 = Pc0;
        Pc0 = Pn0;
        Pp1 = Pc1;
        Pc1 = Pn1;
        CZp = CZ;
        zo = zno;
    }
}

// Items of a round: item = tile * pairs + pair, pair q = sorted samples 2q and
// 2q + 1 (tile-major, as k_population8).
template <int LR, int MINB>
__global__ void __launch_bounds__(256, MINB) k_population9(PopArgs p) {
    const int maxsteps = p.S > 0 ? p.rec[0].nsteps : 0;
    int active = p.S;
    const int rows = 256 / LR;
    for (int k = 0; k < maxsteps; ++k) {
        while (active > 0 && p.rec[active - 1].nsteps <= k) --active;
        const float *in = (k & 1) ? p.buf1 : p.buf0;
        float *out = (k & 1) ? p.buf0 : p.buf1;
        const unsigned pairs = (unsigned)(active + 1) / 2;
        const unsigned items = pairs * (unsigned)p.tiles;
        for (unsigned it = blockIdx.x; it < items; it += gridDim.x) {
            const unsigned q = it % pairs, t = it / pairs;
            const int r0 = 2 * (int)q, r1 = r0 + 1;
            const bool two = r1 < active;
            const int ty = (int)t % p.tiles_y, tz = (int)t / p.tiles_y;
            const SampleRec &s0 = p.rec[r0];
            const size_t off0 = (size_t)s0.order * p.stride;
            const bool last0 = k == s0.nsteps - 1;
            const float a0 = last0 ? s0.a2 : s0.a, b0 = last0 ? s0.b2 : s0.b;
            size_t off1 = off0;
            float a1 = a0, b1 = b0;
            if (two) {
                const SampleRec &s1 = p.rec[r1];
                off1 = (size_t)s1.order * p.stride;
                const bool last1 = k == s1.nsteps - 1;
                a1 = last1 ? s1.a2 : s1.a;
                b1 = last1 ? s1.b2 : s1.b;
            }
            march_tile_pair<LR>(p.n, p.TZ, ty * rows, tz * p.TZ, two, in + off0, out + off0, in + off1,
                                out + off1, p.cxs, p.cy, p.cz, a0, b0, a1, b1);
        }
        if (k + 1 < maxsteps && !grid_barrier(p.barrier, p.status, gridDim.x)) return;
    }
}

// ---- population kernel, bulk-copy (TMA) staged ---------------------------------
// Same arithmetic and operation order as march_tile_s. A producer warp
// copies each z-plane of a tile into a ring of D shared-memory slots with
// cp.async.bulk (the TMA unit; mbarriers per slot, completion by byte
// count), up to D planes ahead of the plane being computed, so a CTA keeps
// D planes of loads in flight without holding registers for them. A slot
// holds, for one plane: density rows y0-1 .. y0+RY (periodic), cy rows
// y0-1 .. y0+RY-1 and cx, cz, mask rows y0 .. y0+RY-1 (8 copies, rows of
// n floats; the RY-row blocks are contiguous in memory). Every wait is
// bounded; on a timeout the kernel records DEV_COPY_TIMEOUT, waits (bounded)
// for the copies it has in flight and leaves.
__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// bounded wait for the given phase parity; false on timeout
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity) {
    const unsigned addr = smem_u32(bar);
    for (long long spins = 0; spins < (1ll << 24); ++spins) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
        if (spins > 64) __nanosleep(32);
    }
    return false;
}

template <int LR, int RY, int D>
struct TmaRing {
    static constexpr int n = 4 * LR;
    static constexpr int ROW = n * 4;                  // bytes per row
    static constexpr int DEN = (RY + 2) * n;           // floats: density rows y0-1 .. y0+RY
    static constexpr int CYR = (RY + 1) * n;           // cy rows y0-1 .. y0+RY-1
    static constexpr int BLK = RY * n;                 // cx, cz, mask rows y0 .. y0+RY-1
    static constexpr int SLOT = DEN + CYR + 3 * BLK;   // floats per slot
    static constexpr unsigned BYTES = SLOT * 4;
    static constexpr size_t smem() { return (size_t)D * BYTES + 64 * D; }
};

// Warp-specialised variant of the bulk-copy family: warp NC (after the NC
// consumer warps) produces, the consumer warps compute. Each slot has a
// "full" barrier (completed by the copies' byte count) and an "empty"
// barrier (one arrival per consumer warp once the plane is no longer read),
// so consumers never synchronise as a block: a consumer warp waits only for
// the planes it reads, the producer only for a slot to be released. All
// waits are bounded; a timeout sets a shared flag and the status word, and
// every warp leaves at its next wait.
template <int LR, int RY, int D, int MINB>
__global__ void __launch_bounds__(LR *RY + 32, MINB) k_population6(PopArgs p) {
    using R = TmaRing<LR, RY, D>;
    constexpr int n = R::n;
    constexpr int plane = n * n;
    constexpr int NC = LR * RY / 32;  // consumer warps
    extern __shared__ __align__(128) float smem6[];
    float *ring = smem6;
    unsigned long long *full = reinterpret_cast<unsigned long long *>(smem6 + (size_t)D * R::SLOT);
    unsigned long long *empty = full + D;
    __shared__ int abort_flag;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool producer = warp == NC;
    if (threadIdx.x == 0) {
        for (int i = 0; i < D; ++i) {
            mbar_init(full + i, 1);
            mbar_init(empty + i, NC);
        }
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    auto fail = [&]() {
        atomicExch(&abort_flag, 1);
        atomicExch(p.status, (int)DEV_COPY_TIMEOUT);
    };
    const int r = producer ? 0 : threadIdx.x / LR, li = threadIdx.x % LR, x0 = 4 * li;
    int slot = 0;
    unsigned phase = 0;  // this warp's cursor: next plane's slot and full/empty phase
    unsigned used = 0, last_phase = 0;  // producer: per-slot latest copy (drain)
    const int maxsteps = p.S > 0 ? p.rec[0].nsteps : 0;
    const int nplanes = p.TZ + 2;
    int active = p.S;
    long long q = 0;  // plane sequence number of the next plane (both roles)
    for (int k = 0; k < maxsteps; ++k) {
        while (active > 0 && p.rec[active - 1].nsteps <= k) --active;
        const float *in = (k & 1) ? p.buf1 : p.buf0;
        float *out = (k & 1) ? p.buf0 : p.buf1;
        const int items = active * p.tiles;
        const int my_items = (int)blockIdx.x < items ? (items - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
        for (int m = 0; m < my_items; ++m) {
            const int it = (int)blockIdx.x + m * (int)gridDim.x;
            const int smp = it % active, t = it / active;
            const int y0 = (t % p.tiles_y) * RY, tz0 = (t / p.tiles_y) * p.TZ;
            const size_t off = (size_t)p.rec[smp].order * p.stride;
            if (producer) {
                for (int j = 0; j < nplanes; ++j, ++q) {
                    if (lane == 0 && !*(volatile int *)&abort_flag) {
                        // the slot's previous plane (q - D) released by every consumer warp
                        if (q >= D && !mbar_wait(empty + slot, phase ^ 1u)) fail();
                        if (!*(volatile int *)&abort_flag) {
                            unsigned long long *mb = full + slot;
                            float *dst = ring + (size_t)slot * R::SLOT;
                            int zz = tz0 - 1 + j;
                            zz = zz < 0 ? zz + n : (zz >= n ? zz - n : zz);
                            const int ym = y0 == 0 ? n - 1 : y0 - 1, yp = y0 + RY == n ? 0 : y0 + RY;
                            const float *pl = in + off + (size_t)zz * plane;
                            const size_t ao = (size_t)zz * plane;
                            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                            mbar_expect_tx(mb, R::BYTES);
                            bulk_g2s(dst, pl + (size_t)ym * n, R::ROW, mb);
                            bulk_g2s(dst + n, pl + (size_t)y0 * n, RY * R::ROW, mb);
                            bulk_g2s(dst + (RY + 1) * n, pl + (size_t)yp * n, R::ROW, mb);
                            float *cyb = dst + R::DEN;
                            bulk_g2s(cyb, p.cy + ao + (size_t)ym * n, R::ROW, mb);
                            bulk_g2s(cyb + n, p.cy + ao + (size_t)y0 * n, RY * R::ROW, mb);
                            float *cxb = cyb + R::CYR, *czb = cxb + R::BLK, *mkb = czb + R::BLK;
                            bulk_g2s(cxb, p.cx + ao + (size_t)y0 * n, RY * R::ROW, mb);
                            bulk_g2s(czb, p.cz + ao + (size_t)y0 * n, RY * R::ROW, mb);
                            bulk_g2s(mkb, p.msk + ao + (size_t)y0 * n, RY * R::ROW, mb);
                            used |= 1u << slot;
                            last_phase = (last_phase & ~(1u << slot)) | (phase << slot);
                        }
                    }
                    if (++slot == D) {
                        slot = 0;
                        phase ^= 1u;
                    }
                }
                continue;
            }
            // consumers
            const bool last = k == p.rec[smp].nsteps - 1;
            const float a = last ? p.rec[smp].a2 : p.rec[smp].a;
            const float b = last ? p.rec[smp].b2 : p.rec[smp].b;
            const int y = y0 + r;
            auto advance = [&]() {
                if (++slot == D) {
                    slot = 0;
                    phase ^= 1u;
                }
                ++q;
            };
            auto release = [&](int sl) {  // this warp no longer reads slot sl
                __syncwarp();
                if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(empty + sl)) : "memory");
            };
            // planes j = 0 (z = tz0 - 1) and j = 1 (z = tz0)
            const int s0 = slot;
            if (!mbar_wait(full + slot, phase)) fail();
            advance();
            int sc = slot;
            if (!mbar_wait(full + slot, phase)) fail();
            advance();
            if (*(volatile int *)&abort_flag) break;
            const float *b0 = ring + (size_t)s0 * R::SLOT;
            float4 Pp = *reinterpret_cast<const float4 *>(b0 + (r + 1) * n + x0);
            float4 CZp = *reinterpret_cast<const float4 *>(b0 + R::DEN + R::CYR + R::BLK + r * n + x0);
            float4 Pc = *reinterpret_cast<const float4 *>(ring + (size_t)sc * R::SLOT + (r + 1) * n + x0);
            release(s0);
            for (int dz = 0; dz < p.TZ; ++dz) {
                const int z = tz0 + dz;
                const int sn = slot;  // plane z + 1
                if (!mbar_wait(full + slot, phase)) fail();
                advance();
                if (*(volatile int *)&abort_flag) break;
                const float *pc = ring + (size_t)sc * R::SLOT, *pn = ring + (size_t)sn * R::SLOT;
                const float4 Pn = *reinterpret_cast<const float4 *>(pn + (r + 1) * n + x0);
                const float4 PS = *reinterpret_cast<const float4 *>(pc + r * n + x0);
                const float4 PN = *reinterpret_cast<const float4 *>(pc + (r + 2) * n + x0);
                const float *cyb = pc + R::DEN, *cxb = cyb + R::CYR, *czb = cxb + R::BLK, *mkb = czb + R::BLK;
                const float4 CYm = *reinterpret_cast<const float4 *>(cyb + r * n + x0);
                const float4 CY = *reinterpret_cast<const float4 *>(cyb + (r + 1) * n + x0);
                const float4 CX = *reinterpret_cast<const float4 *>(cxb + r * n + x0);
                const float4 CZ = *reinterpret_cast<const float4 *>(czb + r * n + x0);
                const float4 M = *reinterpret_cast<const float4 *>(mkb + r * n + x0);
                release(sc);  // plane z is read for the last time above
                const float left = __shfl_sync(0xffffffffu, Pc.w, (li + LR - 1) % LR, LR);
                const float right = __shfl_sync(0xffffffffu, Pc.x, (li + 1) % LR, LR);
                const float cxl = __shfl_sync(0xffffffffu, CX.w, (li + LR - 1) % LR, LR);
                const float pv[6] = {left, Pc.x, Pc.y, Pc.z, Pc.w, right};
                const float cxa[5] = {cxl, CX.x, CX.y, CX.z, CX.w};
                const float ps[4] = {PS.x, PS.y, PS.z, PS.w}, pnn[4] = {PN.x, PN.y, PN.z, PN.w};
                const float pp[4] = {Pp.x, Pp.y, Pp.z, Pp.w}, pq[4] = {Pn.x, Pn.y, Pn.z, Pn.w};
                const float cy4[4] = {CY.x, CY.y, CY.z, CY.w}, cym4[4] = {CYm.x, CYm.y, CYm.z, CYm.w};
                const float cz4[4] = {CZ.x, CZ.y, CZ.z, CZ.w}, czp4[4] = {CZp.x, CZp.y, CZp.z, CZp.w};
                const float m4[4] = {M.x, M.y, M.z, M.w};
                float o[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float f0 = pv[i + 1];
                    float lap = cxa[i] * (pv[i] - f0);
                    lap = fmaf(cxa[i + 1], pv[i + 2] - f0, lap);
                    lap = fmaf(cym4[i], ps[i] - f0, lap);
                    lap = fmaf(cy4[i], pnn[i] - f0, lap);
                    lap = fmaf(czp4[i], pp[i] - f0, lap);
                    lap = fmaf(cz4[i], pq[i] - f0, lap);
                    float v = fmaf(a, lap, f0);
                    v = fmaf(b * f0, 1.0f - f0, v);
                    v = fminf(fmaxf(v, 0.0f), 1.0f);
                    o[i] = m4[i] != 0.0f ? v : 0.0f;
                }
                __stcg(reinterpret_cast<float4 *>(out + off + (size_t)x0 + (size_t)n * y + (size_t)plane * z),
                       make_float4(o[0], o[1], o[2], o[3]));
                Pp = Pc;
                Pc = Pn;
                CZp = CZ;
                sc = sn;
            }
            if (*(volatile int *)&abort_flag) break;
            release(sc);  // plane tz0 + TZ (j = TZ + 1): read as z + 1 only
        }
        // this round's stores before the next round's bulk copies read them
        asm volatile("fence.proxy.async.global;\n" ::: "memory");
        __syncthreads();
        if (*(volatile int *)&abort_flag) break;
        if (k + 1 < maxsteps && !grid_barrier(p.barrier, p.status, gridDim.x)) return;
        asm volatile("fence.proxy.async.global;\n" ::: "memory");
    }
    if (abort_flag && producer && lane == 0) {
        // let this CTA's copies in flight land (bounded) before leaving; if one
        // of these waits gives up too, copies may still be writing this CTA's
        // shared memory when it exits, and the host is told so apart from the
        // ordinary timeout
        for (int sl = 0; sl < D; ++sl)
            if ((used >> sl & 1u) && !mbar_wait(full + sl, last_phase >> sl & 1u))
                atomicExch(p.status, (int)DEV_DRAIN_TIMEOUT);
    }
}

// ---- population kernel, two time steps per sweep (temporal blocking) -------------
// A CTA of 10 warps owns a tile of 8 rows (y0 .. y0+7) x TZ planes. Warp w
// computes the first step for row y0-1+w (the tile's rows and one halo row
// on each side) while marching z from tz0-1 to tz0+TZ, with the same
// per-cell operation sequence as march_tile_s; the first-step rows go through a
// 3-plane ring in shared memory, from which warps 1..8 compute the second
// step of plane z-1 (own row's z-2, z-1, z in registers, rows y-1 and y+1
// from the ring, x-neighbours by shuffle). Each round advances every active
// sample by two steps (one when a single step is left), so phi is read and
// written once per two steps. Rounds alternate the buffers; a sample starts
// in buffer (nsteps / 2) & 1 (k_gaussian_ic) and ends in nsteps & 1.
// RELOAD: the second step re-reads its cell's anatomy (an L1/L2 hit: the
// warp read it one plane earlier) instead of carrying it in registers.
template <int MINB, bool RELOAD>
__global__ void __launch_bounds__(320, MINB) k_population7(PopArgs p) {
    constexpr int LR = 32, n = 128, RY = 8, NW = RY + 2;
    constexpr size_t plane = (size_t)n * n;
    __shared__ __align__(16) float ring[3][NW][n];
    const int w = threadIdx.x / LR, li = threadIdx.x % LR, x0 = 4 * li;
    const int maxsteps = p.S > 0 ? p.rec[0].nsteps : 0;
    const int rounds = (maxsteps + 1) / 2;
    int active = p.S;
    for (int j = 0; j < rounds; ++j) {
        const int k = 2 * j;  // first step of the round
        while (active > 0 && p.rec[active - 1].nsteps <= k) --active;
        const long items = (long)active * p.tiles;
        for (long it = blockIdx.x; it < items; it += gridDim.x) {
            const int r = (int)(it % active), t = (int)(it / active);
            const SampleRec rec = p.rec[r];
            const int y0 = (t % p.tiles_y) * RY, tz0 = (t / p.tiles_y) * p.TZ;
            const bool two = rec.nsteps - k >= 2;
            const bool last1 = k == rec.nsteps - 1, last2 = k + 1 == rec.nsteps - 1;
            const float a1 = last1 ? rec.a2 : rec.a, b1 = last1 ? rec.b2 : rec.b;
            const float a2 = last2 ? rec.a2 : rec.a, b2 = last2 ? rec.b2 : rec.b;
            const int s0 = (rec.nsteps / 2) & 1;
            const float *in = (((j + s0) & 1) ? p.buf1 : p.buf0) + (size_t)rec.order * p.stride;
            float *out = (((j + s0) & 1) ? p.buf0 : p.buf1) + (size_t)rec.order * p.stride;
            const int y = (y0 - 1 + w + n) % n;        // this warp's first-step row
            const int ym = y == 0 ? n - 1 : y - 1, yp = y == n - 1 ? 0 : y + 1;
            const bool inner = w >= 1 && w <= RY;      // rows of the tile (second step, output)
            auto at = [&](int yy, int zz) -> unsigned { return (unsigned)(x0 + n * yy) + (unsigned)plane * (unsigned)zz; };
            auto wz = [&](int zz) { return zz < 0 ? zz + n : (zz >= n ? zz - n : zz); };
            // first-step state: planes z-1, z in registers; anatomy carried for the second step
            const int zstart = tz0 - 1;
            float4 Pp = __ldcg(reinterpret_cast<const float4 *>(in + at(y, wz(zstart - 1))));
            float4 Pc = __ldcg(reinterpret_cast<const float4 *>(in + at(y, wz(zstart))));
            float4 CZp = __ldg(reinterpret_cast<const float4 *>(p.cz + at(y, wz(zstart - 1))));
            // second-step inputs of this row: first-step values of planes z-2, z-1
            float4 Q2 = make_float4(0, 0, 0, 0), Q1 = Q2;
            // anatomy of plane z-1 of this row (the second step's cell), and cz of z-2
            float4 AX = Q2, AY = Q2, AYm = Q2, AZ = Q2, AM = Q2, AZp = Q2;
            for (int step = 0; step < p.TZ + 2; ++step) {
                const int z = wz(zstart + step);
                const int zn = wz(zstart + step + 1);
                // ---- first step, plane z, row y ----
                const float4 Pn = __ldcg(reinterpret_cast<const float4 *>(in + at(y, zn)));
                const float4 PS = __ldcg(reinterpret_cast<const float4 *>(in + at(ym, z)));
                const float4 PN = __ldcg(reinterpret_cast<const float4 *>(in + at(yp, z)));
                const float4 CX = __ldg(reinterpret_cast<const float4 *>(p.cx + at(y, z)));
                const float4 CY = __ldg(reinterpret_cast<const float4 *>(p.cy + at(y, z)));
                const float4 CYm = __ldg(reinterpret_cast<const float4 *>(p.cy + at(ym, z)));
                const float4 CZ = __ldg(reinterpret_cast<const float4 *>(p.cz + at(y, z)));
                const float4 M = __ldg(reinterpret_cast<const float4 *>(p.msk + at(y, z)));
                float4 F;
                {
                    const float left = __shfl_sync(0xffffffffu, Pc.w, (li + LR - 1) % LR, LR);
                    const float right = __shfl_sync(0xffffffffu, Pc.x, (li + 1) % LR, LR);
                    const float cxl = __shfl_sync(0xffffffffu, CX.w, (li + LR - 1) % LR, LR);
                    const float pv[6] = {left, Pc.x, Pc.y, Pc.z, Pc.w, right};
                    const float cxa[5] = {cxl, CX.x, CX.y, CX.z, CX.w};
                    const float ps[4] = {PS.x, PS.y, PS.z, PS.w}, pn[4] = {PN.x, PN.y, PN.z, PN.w};
                    const float pp[4] = {Pp.x, Pp.y, Pp.z, Pp.w}, pq[4] = {Pn.x, Pn.y, Pn.z, Pn.w};
                    const float cy4[4] = {CY.x, CY.y, CY.z, CY.w}, cym4[4] = {CYm.x, CYm.y, CYm.z, CYm.w};
                    const float cz4[4] = {CZ.x, CZ.y, CZ.z, CZ.w}, czp4[4] = {CZp.x, CZp.y, CZp.z, CZp.w};
                    const float m4[4] = {M.x, M.y, M.z, M.w};
                    float o[4];
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const float f0 = pv[i + 1];
                        float lap = cxa[i] * (pv[i] - f0);
                        lap = fmaf(cxa[i + 1], pv[i + 2] - f0, lap);
                        lap = fmaf(cym4[i], ps[i] - f0, lap);
                        lap = fmaf(cy4[i], pn[i] - f0, lap);
                        lap = fmaf(czp4[i], pp[i] - f0, lap);
                        lap = fmaf(cz4[i], pq[i] - f0, lap);
                        float v = fmaf(a1, lap, f0);
                        v = fmaf(b1 * f0, 1.0f - f0, v);
                        v = fminf(fmaxf(v, 0.0f), 1.0f);
                        o[i] = m4[i] != 0.0f ? v : 0.0f;
                    }
                    F = make_float4(o[0], o[1], o[2], o[3]);
                }
                const int zo = zstart + step;  // unwrapped plane of F
                if (!two) {
                    // one step left: the first step is the output
                    if (inner && zo >= tz0 && zo < tz0 + p.TZ)
                        __stcg(reinterpret_cast<float4 *>(out + at(y, z)), F);
                } else {
                    *reinterpret_cast<float4 *>(&ring[step % 3][w][x0]) = F;
                }
                __syncthreads();
                // ---- second step, plane z-1 (unwrapped zo-1), rows of the tile ----
                if (two && step >= 2 && inner) {
                    const int zc = wz(zo - 1);
                    if (RELOAD) {
                        AX = __ldg(reinterpret_cast<const float4 *>(p.cx + at(y, zc)));
                        AY = __ldg(reinterpret_cast<const float4 *>(p.cy + at(y, zc)));
                        AYm = __ldg(reinterpret_cast<const float4 *>(p.cy + at(ym, zc)));
                        AZ = __ldg(reinterpret_cast<const float4 *>(p.cz + at(y, zc)));
                        AZp = __ldg(reinterpret_cast<const float4 *>(p.cz + at(y, wz(zo - 2))));
                        AM = __ldg(reinterpret_cast<const float4 *>(p.msk + at(y, zc)));
                    }
                    const float4 S1 = *reinterpret_cast<const float4 *>(&ring[(step - 1) % 3][w - 1][x0]);
                    const float4 N1 = *reinterpret_cast<const float4 *>(&ring[(step - 1) % 3][w + 1][x0]);
                    const float left = __shfl_sync(0xffffffffu, Q1.w, (li + LR - 1) % LR, LR);
                    const float right = __shfl_sync(0xffffffffu, Q1.x, (li + 1) % LR, LR);
                    const float cxl = __shfl_sync(0xffffffffu, AX.w, (li + LR - 1) % LR, LR);
                    const float pv[6] = {left, Q1.x, Q1.y, Q1.z, Q1.w, right};
                    const float cxa[5] = {cxl, AX.x, AX.y, AX.z, AX.w};
                    const float ps[4] = {S1.x, S1.y, S1.z, S1.w}, pn[4] = {N1.x, N1.y, N1.z, N1.w};
                    const float pp[4] = {Q2.x, Q2.y, Q2.z, Q2.w}, pq[4] = {F.x, F.y, F.z, F.w};
                    const float cy4[4] = {AY.x, AY.y, AY.z, AY.w}, cym4[4] = {AYm.x, AYm.y, AYm.z, AYm.w};
                    const float cz4[4] = {AZ.x, AZ.y, AZ.z, AZ.w}, czp4[4] = {AZp.x, AZp.y, AZp.z, AZp.w};
                    const float m4[4] = {AM.x, AM.y, AM.z, AM.w};
                    float o[4];
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const float f0 = pv[i + 1];
                        float lap = cxa[i] * (pv[i] - f0);
                        lap = fmaf(cxa[i + 1], pv[i + 2] - f0, lap);
                        lap = fmaf(cym4[i], ps[i] - f0, lap);
                        lap = fmaf(cy4[i], pn[i] - f0, lap);
                        lap = fmaf(czp4[i], pp[i] - f0, lap);
                        lap = fmaf(cz4[i], pq[i] - f0, lap);
                        float v = fmaf(a2, lap, f0);
                        v = fmaf(b2 * f0, 1.0f - f0, v);
                        v = fminf(fmaxf(v, 0.0f), 1.0f);
                        o[i] = m4[i] != 0.0f ? v : 0.0f;
                    }
                    __stcg(reinterpret_cast<float4 *>(out + at(y, zc)), make_float4(o[0], o[1], o[2], o[3]));
                }
                // shift: this plane's first-step values and anatomy serve the next
                // iteration's second step (its cell plane is this z)
                Q2 = Q1;
                Q1 = F;
                if (!RELOAD) {
                    AZp = AZ;
                    AX = CX;
                    AY = CY;
                    AYm = CYm;
                    AZ = CZ;
                    AM = M;
                }
                Pp = Pc;
                Pc = Pn;
                CZp = CZ;
            }
        }
        if (j + 1 < rounds && !grid_barrier(p.barrier, p.status, gridDim.x)) return;
    }
}

int grid_for(const Handle &h, size_t work) {
    const size_t blocks = (work + 255) / 256;
    const size_t cap = (size_t)h.num_sms * 8;
    return (int)(blocks < cap ? blocks : cap);
}

// Lanes per row for the supported fast-path sizes.
int lanes_per_row(int n) {
    if (n == 32 || n == 64 || n == 128) return n / 4;
    return 0;
}

struct PopVariant {
    const void *fn;
    int ry, g, threads, tz;
    size_t smem;
    bool tb = false;  // two steps per round (start buffer per sample, see k_gaussian_ic)
    bool skip = false;  // visits only tiles that can be nonzero (needs the batched solver's set-up)
    bool counts = false;  // counts the tiles it computes (gbg_last_population_cells)
    char name[64] = {0};  // kernel and template arguments, plus the tile depth
};

template <int LR, int MINB, bool SLOT = false>
PopVariant make_signmask_variant(int tz) {
    PopVariant v;
    v.fn = (const void *)k_population8<LR, MINB, SLOT>;
    v.ry = 256 / LR;
    v.g = 1;
    v.threads = 256;
    v.tz = tz;
    v.smem = 0;
    v.counts = true;
    std::snprintf(v.name, sizeof(v.name), "k_population8<%d,%d> TZ %d", LR, MINB, tz);
    return v;
}

template <int LR, int MINB, bool SLOT = false>
PopVariant make_skip_variant(int tz) {
    PopVariant v;
    v.fn = (const void *)k_population10<LR, MINB, SLOT>;
    v.ry = 256 / LR;
    v.g = 1;
    v.threads = 256;
    v.tz = tz;
    v.smem = 0;
    v.skip = true;
    v.counts = true;
    std::snprintf(v.name, sizeof(v.name), "k_population10<%d,%d> TZ %d", LR, MINB, tz);
    return v;
}

template <int LR, int MINB>
PopVariant make_pair_variant(int tz) {
    PopVariant v;
    v.fn = (const void *)k_population9<LR, MINB>;
    v.ry = 256 / LR;
    v.g = 2;
    v.threads = 256;
    v.tz = tz;
    v.smem = 0;
    std::snprintf(v.name, sizeof(v.name), "k_population9<%d,%d> TZ %d", LR, MINB, tz);
    return v;
}

template <int MINB, bool RELOAD>
PopVariant make_tb_variant(int tz) {
    PopVariant v;
    v.fn = (const void *)k_population7<MINB, RELOAD>;
    v.ry = 8;
    v.g = 1;
    v.threads = 320;
    v.tz = tz;
    v.smem = 0;
    v.tb = true;
    std::snprintf(v.name, sizeof(v.name), "k_population7<%d,%d> TZ %d", MINB, (int)RELOAD, tz);
    return v;
}

template <int LR, int RY, int D, int MINB>
PopVariant make_ws_variant(int tz) {
    PopVariant v;
    v.fn = (const void *)k_population6<LR, RY, D, MINB>;
    v.ry = RY;
    v.g = 1;
    v.threads = LR * RY + 32;
    v.tz = tz;
    v.smem = TmaRing<LR, RY, D>::smem();
    std::snprintf(v.name, sizeof(v.name), "k_population6<%d,%d,%d,%d> TZ %d", LR, RY, D, MINB, tz);
    return v;
}

// Candidate shapes per grid size; index 0 is the default. The batched solver
// runs the skipping kernel by default; paths without its set-up (the single
// solve) run the first dense register variant instead (dense_default).
int variants_for(int n, PopVariant *out) {
    int k = 0;
    switch (n) {
        case 128:
            out[k++] = make_skip_variant<32, 4>(8);
            out[k++] = make_skip_variant<32, 4>(16);
            out[k++] = make_signmask_variant<32, 4>(16);
            out[k++] = make_signmask_variant<32, 4>(32);
            out[k++] = make_signmask_variant<32, 5>(16);
            out[k++] = make_pair_variant<32, 3>(16);
            out[k++] = make_pair_variant<32, 3>(32);
            out[k++] = make_tb_variant<2, true>(32);
            out[k++] = make_ws_variant<32, 8, 3, 3>(32);
            break;
        case 64:
            out[k++] = make_skip_variant<16, 4>(8);
            out[k++] = make_signmask_variant<16, 4>(16);
            out[k++] = make_signmask_variant<16, 5>(16);
            break;
        case 32:
            out[k++] = make_skip_variant<8, 4>(8);
            out[k++] = make_signmask_variant<8, 4>(8);
            break;
    }
    return k;
}

// the kernels keeping every state (population_steps' slot mode): the dense
// default's shape, or the skipping kernel with tile depth tz
PopVariant slot_variant(int n, bool skip, int tz) {
    if (skip) switch (n) {
            case 128:
                return make_skip_variant<32, 4, true>(tz);
            case 64:
                return make_skip_variant<16, 4, true>(tz);
            default:
                return make_skip_variant<8, 4, true>(tz);
        }
    switch (n) {
        case 128:
            return make_signmask_variant<32, 4, true>(16);
        case 64:
            return make_signmask_variant<16, 4, true>(16);
        default:
            return make_signmask_variant<8, 4, true>(8);
    }
}

// index of the first variant that is neither temporally blocked nor skipping
int dense_default(const PopVariant *vs, int nv) {
    for (int i = 0; i < nv; ++i)
        if (!vs[i].tb && !vs[i].skip) return i;
    return 0;
}

int launch_population_v(Handle &h, PopArgs &a, const PopVariant &v) {
    GBG_CUDA_TRY(cudaFuncSetAttribute(v.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)v.smem));
    int bps = 0;
    GBG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, v.fn, v.threads, v.smem));
    if (bps <= 0) {
        set_error("population kernel cannot be resident");
        return GBG_ERR_CUDA;
    }
    const long maxitems = (long)((a.S + v.g - 1) / v.g) * a.tiles;
    long grid = (long)bps * h.num_sms;
    if (grid > maxitems) grid = maxitems;
    if (grid < 1) grid = 1;
    // barrier count and generation, and the visited-tile counter after them
    GBG_CUDA_TRY(cudaMemsetAsync(a.barrier, 0, 4 * sizeof(unsigned), h.stream));
    h.pop_tile_cells = v.counts ? (long long)v.ry * v.tz * a.n : 0;
    void *args[] = {&a};
    // inside a stream capture the events become record nodes of the graph
    // (recorded at each replay), so gbg_last_population_ms times replays too
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    GBG_CUDA_TRY(cudaStreamIsCapturing(h.stream, &cap));
    const unsigned evf = cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
    GBG_CUDA_TRY(cudaEventRecordWithFlags(h.ev_pop[0], h.stream, evf));
    GBG_CUDA_TRY(cudaLaunchCooperativeKernel(v.fn, dim3((unsigned)grid), dim3(v.threads), args, v.smem,
                                             h.stream));
    GBG_CUDA_TRY(cudaEventRecordWithFlags(h.ev_pop[1], h.stream, evf));
    h.ev_pop_recorded = true;
    h.launches++;
    return GBG_OK;
}

bool variant_is_tb(const Handle &h) {
    PopVariant vs[32];
    const int nv = variants_for(h.n, vs);
    const int vi = h.pop_variant;
    return vi >= 0 && vi < nv && vs[vi].tb;
}

bool variant_is_skip(const Handle &h) {
    PopVariant vs[32];
    const int nv = variants_for(h.n, vs);
    const int vi = h.pop_variant;
    return vi >= 0 && vi < nv && vs[vi].skip;
}

// Live-tile list of the skipping kernel for tiles of rows x tz cells, built
// from the fast tables' mask (sign bit of cxs) and kept until the anatomy
// changes or another tile shape is asked for.
int ensure_live_tiles(Handle &h, int rows, int tz) {
    if (h.live_valid && h.live_ry == rows && h.live_tz == tz) return GBG_OK;
    ++h.state_gen;
    const int tiles = (h.n / rows) * (h.n / tz);
    if (!h.tile_live) {
        // sized for the smallest tiles any variant uses (rows >= 8, tz >= 8)
        const size_t cap = (size_t)(h.n / 8 + 1) * (size_t)(h.n / 8 + 1);
        GBG_CUDA_TRY(cudaMalloc((void **)&h.tile_live, cap));
        GBG_CUDA_TRY(cudaMalloc((void **)&h.live_list, cap * sizeof(int)));
        GBG_CUDA_TRY(cudaMalloc((void **)&h.live_count, sizeof(int)));
    }
    k_tile_live<<<tiles, 256, 0, h.stream>>>(h.n, rows, tz, h.cxs, h.tile_live);
    k_compact_live<<<1, 32, 0, h.stream>>>(tiles, h.tile_live, h.live_list, h.live_count);
    h.launches += 2;
    GBG_CUDA_TRY(cudaGetLastError());
    h.live_valid = true;
    h.live_ry = rows;
    h.live_tz = tz;
    return GBG_OK;
}

// allow_tb = false (the single-solve path, whose state must start in buf0)
// runs the default variant in place of a temporally blocked one; allow_skip =
// false (any path but the batched solver, which sets up the initial-support
// boxes and the zero-filled second buffer) runs it in place of the skipping
// kernel
int launch_population(Handle &h, float *buf0, float *buf1, const SampleRec *rec_sorted, int S,
                      bool allow_tb = true, bool allow_skip = false, size_t slot = 0,
                      const int *box = nullptr, int grow0 = 0) {
    const int LR = lanes_per_row(h.n);
    if (!LR) {
        set_error("fast path supports n = 32, 64 or 128");
        return GBG_ERR_UNSUPPORTED;
    }
    PopVariant vs[32];
    const int nv = variants_for(h.n, vs);
    int vi = h.pop_variant;
    if (vi < 0 || vi >= nv || (vs[vi].tb && !allow_tb) || (vs[vi].skip && !allow_skip))
        vi = dense_default(vs, nv);
    // slot mode: the skipping kernel when boxes are given, at the chosen
    // skipping shape's tile depth (the default one's otherwise)
    const int slot_tz = (h.pop_variant >= 0 && h.pop_variant < nv && vs[h.pop_variant].skip) ? vs[h.pop_variant].tz
                                                                                            : vs[0].tz;
    const PopVariant v = slot ? slot_variant(h.n, box != nullptr, slot_tz) : vs[vi];
    PopArgs a;
    a.n = h.n;
    a.S = S;
    a.TZ = v.tz;
    a.tiles_y = h.n / v.ry;
    a.tiles = a.tiles_y * (h.n / a.TZ);
    a.stride = h.N;
    a.buf0 = buf0;
    a.buf1 = buf1;
    a.slot = slot;
    a.cx = h.cx;
    a.cy = h.cy;
    a.cz = h.cz;
    a.msk = h.msk;
    a.cxs = h.cxs;
    a.rec = rec_sorted;
    a.barrier = h.barrier;
    a.status = h.dev_status;
    a.live_list = nullptr;
    a.live_count = nullptr;
    a.tile_live = nullptr;
    a.box = nullptr;
    a.grow0 = grow0;
    a.visited = reinterpret_cast<unsigned long long *>(h.barrier + 2);
    if (v.skip) {
        if (h.n % v.tz || h.n % v.ry) {
            set_error("tile shape does not divide the grid");
            return GBG_ERR_UNSUPPORTED;
        }
        if (int rc = ensure_live_tiles(h, v.ry, v.tz)) return rc;
        a.live_list = h.live_list;
        a.live_count = h.live_count;
        a.tile_live = h.tile_live;
        a.box = box ? box : batch_boxes(h);
    }
    return launch_population_v(h, a, v);
}

}  // namespace

int population_steps(Handle &h, float *buf0, float *buf1, const SampleRec *recs, SampleRec *sorted, int *rank,
                     int S, size_t slot, const int *box, int grow0) {
    if (!lanes_per_row(h.n)) {
        set_error("fast path supports n = 32, 64 or 128");
        return GBG_ERR_UNSUPPORTED;
    }
    if (int rc = fast_build_tables(h, (double)0.1f)) return rc;
    k_sort_schedule<<<(S + 127) / 128, 128, 0, h.stream>>>(recs, S, sorted, rank);
    h.launches++;
    GBG_CUDA_TRY(cudaGetLastError());
    return launch_population(h, buf0, buf1, sorted, S, false, box != nullptr, slot, box, grow0);
}

bool population_supported(int n) { return lanes_per_row(n) != 0; }

int population_variant_count(int n) {
    PopVariant vs[32];
    return variants_for(n, vs);
}

int population_variant_name(int n, int vi, char *buf, int len) {
    PopVariant vs[32];
    const int nv = variants_for(n, vs);
    if (vi < 0 || vi >= nv || !buf || len < 1) return GBG_ERR_ARG;
    std::snprintf(buf, (size_t)len, "%s", vs[vi].name);
    return GBG_OK;
}

int population_variant_shape(int n, int vi, int *ry, int *g, int *threads) {
    PopVariant vs[32];
    const int nv = variants_for(n, vs);
    if (vi < 0 || vi >= nv) return GBG_ERR_ARG;
    *ry = vs[vi].ry;
    *g = vs[vi].g;
    *threads = vs[vi].threads;
    return GBG_OK;
}

int check_device_status(Handle &h) {
    int st = 0;
    GBG_CUDA_TRY(cudaMemcpyAsync(&st, h.dev_status, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    if (st != DEV_OK) {
        const int zero = 0;
        cudaMemcpy(h.dev_status, &zero, sizeof(int), cudaMemcpyHostToDevice);
        set_error(st == DEV_COPY_TIMEOUT    ? "device-side bulk copy did not complete"
                  : st == DEV_DRAIN_TIMEOUT ? "device-side bulk copy did not complete, and copies still in "
                                              "flight did not land before the kernel left"
                  : st == DEV_MMA_TIMEOUT   ? "device-side tensor-core MMA did not complete"
                                            : "device-side grid barrier timed out");
        return GBG_ERR_TIMEOUT;
    }
    return GBG_OK;
}

int launch_schedule_smooth(Handle &h, const gbg_sample *samples_device, int S, double L, double dt0,
                           SampleRec *dev_out) {
    k_schedule_smooth<<<(S + 127) / 128, 128, 0, h.stream>>>(samples_device, S, h.n, L, dt0, dev_out);
    h.launches++;
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
}

int launch_gaussian_ic(Handle &h, const gbg_sample *samples_device, int S, double peak, double sigma,
                       float *phi, int *box) {
    k_gaussian_ic<<<ic_grid(h, S), 256, 0, h.stream>>>(h.n, samples_device, S, peak, sigma, h.pw, h.pg, phi,
                                                        nullptr, nullptr, box);
    h.launches++;
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
}

int fast_build_tables(Handle &h, double ratio) {
    if (h.fast_valid && h.fast_ratio == ratio) return GBG_OK;
    ++h.state_gen;
    k_fast_tables<<<grid_for(h, h.N), 256, 0, h.stream>>>(h.n, h.pw, h.pg, ratio, h.cx, h.cy,
                                                           h.cz, h.msk, h.cxs);
    h.launches++;
    GBG_CUDA_TRY(cudaGetLastError());
    h.fast_ratio = ratio;
    h.fast_valid = true;
    return GBG_OK;
}

// Single solve on the fast path: a one-sample population.
int fast_steps_single(Handle &h, double Dw, double rho, double dt, long nsteps) {
    if (nsteps <= 0) return GBG_OK;
    if (nsteps > 100000000L) {
        set_error("nsteps too large");
        return GBG_ERR_ARG;
    }
    const double hh = 1.0 / h.n;
    SampleRec r;
    r.a = (float)(dt * Dw * (1. / (hh * hh)));
    r.b = (float)(dt * rho);
    r.nsteps = (int)nsteps;
    r.order = 0;
    r.dt = dt;
    r.a2 = r.a;
    r.b2 = r.b;
    SampleRec *d_rec = reinterpret_cast<SampleRec *>(h.bwork);
    GBG_CUDA_TRY(cudaMemcpyAsync(d_rec, &r, sizeof(r), cudaMemcpyHostToDevice, h.stream));
    int rc = launch_population(h, (float *)h.phi[h.cur], (float *)h.phi[h.cur ^ 1], d_rec, 1, false);
    if (rc) return rc;
    rc = check_device_status(h);
    if (rc) return rc;
    h.cur ^= (int)(nsteps & 1);
    return GBG_OK;
}

int batch_solve_device(Handle &h, const gbg_sample *samples_device, int S,
                       const gbg_batch_opts &o, gbg_lik_result *loglik_device, long *nsteps_host) {
    if (S <= 0 || S > h.max_samples) {
        set_error("S out of range (1..max_samples)");
        return GBG_ERR_ARG;
    }
    const bool f32ref = h.prec == GBG_PREC_F32REF;
    SampleRec *unsorted = batch_unsorted(h);
    SampleRec *sorted = batch_sorted(h);
    int *rank_of = batch_rank_of(h);
    if (o.dt0 != 0)
        k_schedule_smooth<<<(S + 127) / 128, 128, 0, h.stream>>>(samples_device, S, h.n, o.L, o.dt0, unsorted);
    else
        k_schedule<<<(S + 127) / 128, 128, 0, h.stream>>>(samples_device, S, h.n, o.L, f32ref ? 1 : 0,
                                                          unsorted);
    k_sort_schedule<<<(S + 127) / 128, 128, 0, h.stream>>>(unsorted, S, sorted, rank_of);
    const bool tb = variant_is_tb(h);
    // the skipping kernel: initial-support boxes recorded by the IC kernel and
    // a zero-filled second buffer (it holds zeros wherever a round skips)
    const bool skip = !f32ref && variant_is_skip(h);
    if (skip) {
        GBG_CUDA_TRY(cudaMemsetAsync(batch_boxes(h), 0, (size_t)S * 4 * sizeof(int), h.stream));
        GBG_CUDA_TRY(cudaMemsetAsync(h.bphi[1], 0, (size_t)S * h.N * sizeof(float), h.stream));
    }
    k_gaussian_ic<<<ic_grid(h, S), 256, 0, h.stream>>>(h.n, samples_device, S, o.ic_peak, o.ic_sigma, h.pw,
                                                        h.pg, h.bphi[0], tb ? h.bphi[1] : nullptr,
                                                        tb ? unsorted : nullptr, skip ? batch_boxes(h) : nullptr);
    h.launches += 3;
    GBG_CUDA_TRY(cudaGetLastError());
    if (f32ref) {
        set_error("the batched solver runs on the fast path (GBG_PREC_F32) only");
        return GBG_ERR_UNSUPPORTED;
    }
    int rc = fast_build_tables(h, (double)0.1f);
    if (rc) return rc;
    rc = launch_population(h, h.bphi[0], h.bphi[1], sorted, S, true, skip);
    if (rc) return rc;
    if (o.with_loglik && loglik_device) {
        // final field of sample s sits in buffer (nsteps_s & 1); the likelihood
        // kernel resolves that per sample through the unsorted records.
        rc = lik_evaluate_population(h, h.bphi[0], h.bphi[1], unsorted, S, loglik_device);
        if (rc) return rc;
    }
    if (nsteps_host) {
        std::vector<SampleRec> tmp(S);
        GBG_CUDA_TRY(cudaMemcpyAsync(tmp.data(), unsorted, sizeof(SampleRec) * S,
                                     cudaMemcpyDeviceToHost, h.stream));
        GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
        for (int s = 0; s < S; ++s) nsteps_host[s] = tmp[s].nsteps;
    }
    return GBG_OK;
}

int batch_prepare(Handle &h, int S, const gbg_batch_opts &o) {
    if (h.prec != GBG_PREC_F32) return GBG_OK;  // the eager path reports the error
    if (int rc = fast_build_tables(h, (double)0.1f)) return rc;
    if (variant_is_skip(h)) {
        PopVariant vs[32];
        variants_for(h.n, vs);
        const PopVariant &v = vs[h.pop_variant];
        if (h.n % v.tz == 0 && h.n % v.ry == 0)
            if (int rc = ensure_live_tiles(h, v.ry, v.tz)) return rc;
    }
    if (o.with_loglik)
        if (int rc = lik_reserve(h, S)) return rc;
    return GBG_OK;
}

void batch_graphs_clear(Handle &h) {
    for (BatchGraph &g : h.graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    h.graphs.clear();
}

// Graphs kept per handle; the least recently used is dropped beyond this.
constexpr size_t kMaxBatchGraphs = 8;

int batch_graph_run(Handle &h, const gbg_sample *samples_device, int S, const gbg_batch_opts &o,
                    gbg_lik_result *loglik_device) {
    const int wl = (o.with_loglik && loglik_device) ? 1 : 0;
    auto same = [&](const BatchGraph &g) {
        return g.S == S && g.with_loglik == wl && g.variant == h.pop_variant && g.L == o.L && g.ic_peak == o.ic_peak &&
               g.ic_sigma == o.ic_sigma && g.dt0 == o.dt0 && g.samples == samples_device &&
               g.lik == (const void *)loglik_device;
    };
    BatchGraph *hit = nullptr;
    for (BatchGraph &g : h.graphs)
        if (same(g)) hit = &g;
    if (hit && hit->gen != h.state_gen) {  // stale: drop it
        cudaGraphExecDestroy(hit->exec);
        h.graphs.erase(h.graphs.begin() + (hit - h.graphs.data()));
        hit = nullptr;
    }
    if (!hit) {
        if (int rc = batch_prepare(h, S, o)) return rc;
        const long long l0 = h.launches;
        GBG_CUDA_TRY(cudaStreamBeginCapture(h.stream, cudaStreamCaptureModeThreadLocal));
        const int rc = batch_solve_device(h, samples_device, S, o, loglik_device, nullptr);
        cudaGraph_t graph = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(h.stream, &graph);
        const long long per = h.launches - l0;
        h.launches = l0;
        if (rc || ec != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            if (!rc) set_error(std::string("batched solve capture: ") + cudaGetErrorString(ec));
            return rc ? rc : GBG_ERR_CUDA;
        }
        cudaGraphExec_t exec = nullptr;
        const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) {
            cudaGetLastError();
            set_error(std::string("batched solve graph: ") + cudaGetErrorString(ei));
            return GBG_ERR_CUDA;
        }
        if (h.graphs.size() >= kMaxBatchGraphs) {
            size_t old = 0;
            for (size_t i = 1; i < h.graphs.size(); ++i)
                if (h.graphs[i].last_use < h.graphs[old].last_use) old = i;
            cudaGraphExecDestroy(h.graphs[old].exec);
            h.graphs.erase(h.graphs.begin() + old);
        }
        BatchGraph g;
        g.S = S;
        g.with_loglik = wl;
        g.variant = h.pop_variant;
        g.L = o.L;
        g.ic_peak = o.ic_peak;
        g.ic_sigma = o.ic_sigma;
        g.dt0 = o.dt0;
        g.samples = samples_device;
        g.lik = loglik_device;
        g.gen = h.state_gen;
        g.launches = per;
        g.tile_cells = h.pop_tile_cells;
        g.exec = exec;
        h.graphs.push_back(g);
        hit = &h.graphs.back();
    }
    hit->last_use = ++h.graph_clock;
    GBG_CUDA_TRY(cudaGraphLaunch(hit->exec, h.stream));
    h.launches += hit->launches;
    h.pop_tile_cells = hit->tile_cells;
    h.ev_pop_recorded = true;
    return GBG_OK;
}

}  // namespace gbg
