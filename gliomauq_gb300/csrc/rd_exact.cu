// Bit-faithful step kernels: the reference's operator arithmetic, rounded
// operation by operation as its source writes it.
//
// This translation unit is compiled with -fmad=false so that no a*b+c is
// contracted into a fused multiply-add: every + and * here rounds on its own,
// as it does in the reference (compiled without contraction). Division and
// the float<->double conversions are IEEE round-to-nearest.
//
// Real = double  : the reference built with -D_MRAG_REAL_=double
// Real = float   : the reference's default build, where the lab fields, Dw,
//                  Dg, rho and the brain sums are float and df[], the fluxes
//                  and the update are double
//                  (source/Glioma/Glioma_ReactionDiffusionOperator.h:40-42,155,174-216,258).
#include "gbg_internal.cuh"

namespace gbg {
namespace {

__device__ __forceinline__ int wrapm(int i, int n) { return i == 0 ? n - 1 : i - 1; }
__device__ __forceinline__ int wrapp(int i, int n) { return i == n - 1 ? 0 : i + 1; }

// Per-cell brain sum and the three "+" face diffusivities of the Case2 branch
// (Glioma_ReactionDiffusionOperator.h:174-188):
//   k_c  = (p_w Dw + p_g Dg) / (p_w + p_g)            in Real
//   df   = 2.0 * (1.0 / ((1.0/k_c) + (1.0/k_n)))      in double
// A face to a cell with p_w + p_g == 0 gives k_n = 0/0 = NaN, hence df = NaN:
// the reference's boundary-layer behaviour, reproduced as is. The face shared
// by cells c and c+e is the same value from either side (IEEE + commutes).
template <typename Real>
__global__ void k_build_tables(int n, const double *__restrict__ pw, const double *__restrict__ pg,
                               Real Dw, Real Dg, Real *__restrict__ b0, double *__restrict__ dfx,
                               double *__restrict__ dfy, double *__restrict__ dfz) {
    const size_t N = (size_t)n * n * n;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
         c += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(c % n), y = (int)((c / n) % n), z = (int)(c / ((size_t)n * n));
        const size_t nb[4] = {c, (size_t)wrapp(x, n) + (size_t)n * (y + (size_t)n * z),
                              (size_t)x + (size_t)n * (wrapp(y, n) + (size_t)n * z),
                              (size_t)x + (size_t)n * (y + (size_t)n * wrapp(z, n))};
        double inv[4];
        Real bc = 0;
        for (int k = 0; k < 4; ++k) {
            const Real a = (Real)pw[nb[k]], b = (Real)pg[nb[k]];
            const Real brain = a + b;
            const Real kk = (a * Dw + b * Dg) / brain;
            inv[k] = 1.0 / (double)kk;
            if (k == 0) bc = brain;
        }
        b0[c] = bc;
        dfx[c] = 2.0 * (1.0 / (inv[0] + inv[1]));
        dfy[c] = 2.0 * (1.0 / (inv[0] + inv[2]));
        dfz[c] = 2.0 * (1.0 / (inv[0] + inv[3]));
    }
}

// rho * phi * (1. - phi): (rho*phi) in Real, times (1.0 - phi) in double.
__device__ __forceinline__ double reaction(double rho, double p) { return rho * p * (1. - p); }
__device__ __forceinline__ double reaction(float rho, float p) {
    const float rp = rho * p;
    return (double)rp * (1. - (double)p);
}

// One step: RHS of Glioma_ReactionDiffusionOperator<3> (:148-218), the dphidt
// rounding to Real, and UpdateTumor<3> (:254-261) with std::max / std::min
// clamping (NaN -> 0).
template <typename Real>
__global__ void k_exact_step(int n, const Real *__restrict__ phi, Real *__restrict__ out,
                             const Real *__restrict__ b0, const double *__restrict__ dfx,
                             const double *__restrict__ dfy, const double *__restrict__ dfz,
                             Real rho, double dt, double ih2) {
    const size_t N = (size_t)n * n * n;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
         c += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(c % n), y = (int)((c / n) % n), z = (int)(c / ((size_t)n * n));
        const size_t nn = (size_t)n, plane = nn * nn;
        const size_t cW = c - x + wrapm(x, n), cE = c - x + wrapp(x, n);
        const size_t cS = c + ((size_t)wrapm(y, n) - y) * nn, cN = c + ((size_t)wrapp(y, n) - y) * nn;
        const size_t cB = c + ((size_t)wrapm(z, n) - z) * plane, cF = c + ((size_t)wrapp(z, n) - z) * plane;
        const Real p0 = phi[c];
        const Real pW = phi[cW], pE = phi[cE], pS = phi[cS], pN = phi[cN], pB = phi[cB], pF = phi[cF];
        double df0 = 0.0, df1 = 0.0, df2 = 0.0, df3 = 0.0, df4 = 0.0, df5 = 0.0;
        const Real tissue = b0[c] + p0;
        if (tissue > 0.) {
            df0 = dfx[cW]; df1 = dfx[c];
            df2 = dfy[cS]; df3 = dfy[c];
            df4 = dfz[cB]; df5 = dfz[c];
        }
        // :198-203, in order
        if (df0 == 0 && pW > 0.) df1 *= 2.0;
        if (df1 == 0 && pE > 0.) df0 *= 2.0;
        if (df2 == 0 && pS > 0.) df3 *= 2.0;
        if (df3 == 0 && pN > 0.) df2 *= 2.0;
        if (df4 == 0 && pB > 0.) df5 *= 2.0;
        if (df5 == 0 && pF > 0.) df4 *= 2.0;
        const double fin = ih2 * (df0 * (double)pW + df1 * (double)pE + df2 * (double)pS +
                                  df3 * (double)pN + df4 * (double)pB + df5 * (double)pF);
        const double fout = -((df0 + df1 + df2 + df3 + df4 + df5) * (double)p0 * ih2);
        const double react = reaction(rho, p0);
        const Real dphidt = (Real)(fout + fin + react);
        Real v = (Real)((double)p0 + dt * (double)dphidt);
        v = ((Real)0 < v) ? v : (Real)0;
        v = (v < (Real)1) ? v : (Real)1;
        out[c] = v;
    }
}

int grid_for(const Handle &h) {
    const size_t blocks = (h.N + 255) / 256;
    const size_t cap = (size_t)h.num_sms * 8;
    return (int)(blocks < cap ? blocks : cap);
}

}  // namespace

int exact_build_tables(Handle &h, double Dw, double Dg) {
    if (h.tables_valid && h.tab_Dw == Dw && h.tab_Dg == Dg) return GBG_OK;
    const int g = grid_for(h);
    if (h.prec == GBG_PREC_F64) {
        k_build_tables<double><<<g, 256, 0, h.stream>>>(h.n, h.pw, h.pg, Dw, Dg, (double *)h.b0,
                                                        h.dfx, h.dfy, h.dfz);
    } else {
        k_build_tables<float><<<g, 256, 0, h.stream>>>(h.n, h.pw, h.pg, (float)Dw, (float)Dg,
                                                       (float *)h.b0, h.dfx, h.dfy, h.dfz);
    }
    h.launches++;
    GBG_CUDA_TRY(cudaGetLastError());
    h.tab_Dw = Dw;
    h.tab_Dg = Dg;
    h.tables_valid = true;
    return GBG_OK;
}

int exact_steps(Handle &h, double Dw, double Dg, double rho, double dt, long nsteps) {
    int rc = exact_build_tables(h, Dw, Dg);
    if (rc) return rc;
    const double hh = 1.0 / h.n;
    const double ih2 = 1. / (hh * hh);
    const int g = grid_for(h);
    for (long s = 0; s < nsteps; ++s) {
        void *in = h.phi[h.cur], *out = h.phi[h.cur ^ 1];
        if (h.prec == GBG_PREC_F64) {
            k_exact_step<double><<<g, 256, 0, h.stream>>>(h.n, (const double *)in, (double *)out,
                                                          (const double *)h.b0, h.dfx, h.dfy,
                                                          h.dfz, rho, dt, ih2);
        } else {
            k_exact_step<float><<<g, 256, 0, h.stream>>>(h.n, (const float *)in, (float *)out,
                                                         (const float *)h.b0, h.dfx, h.dfy, h.dfz,
                                                         (float)rho, dt, ih2);
        }
        h.launches++;
        h.cur ^= 1;
    }
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
}

}  // namespace gbg
