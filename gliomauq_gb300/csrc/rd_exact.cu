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

// Tissue tensor of the MALA slopes operator (Glioma_MALA_SlopesOperator.h:131-148):
// inside the tissue (p_w > 0 || p_g > 0), tt[f] = 2/(1/a_c + 1/a_f) with
// a = p_w + p_g * ratioD in double (1/0 = inf gives 0 toward a cell outside
// the tissue), then the Neumann doubling in order; zero outside. Fields are
// read as Real (the reference's cells store p_w, p_g in Real).
template <typename Real>
__global__ void k_mala_tables(int n, const double *__restrict__ pw, const double *__restrict__ pg, double ratio,
                              double *__restrict__ tt) {
    const size_t N = (size_t)n * n * n;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
         c += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(c % n), y = (int)((c / n) % n), z = (int)(c / ((size_t)n * n));
        const size_t nn = (size_t)n, plane = nn * nn;
        const size_t nb[7] = {c,
                              c - x + wrapm(x, n),
                              c - x + wrapp(x, n),
                              c + ((size_t)wrapm(y, n) - y) * nn,
                              c + ((size_t)wrapp(y, n) - y) * nn,
                              c + ((size_t)wrapm(z, n) - z) * plane,
                              c + ((size_t)wrapp(z, n) - z) * plane};
        double t[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        const Real w0 = (Real)pw[c], g0 = (Real)pg[c];
        if (w0 > 0.0 || g0 > 0.0) {
            const double a0 = (double)w0 + (double)g0 * ratio;
            for (int f = 0; f < 6; ++f) {
                const double af = (double)(Real)pw[nb[f + 1]] + (double)(Real)pg[nb[f + 1]] * ratio;
                t[f] = 2.0 * (1.0 / ((1.0 / a0) + (1.0 / af)));
            }
            if (t[0] == 0) t[1] *= 2.0;
            if (t[1] == 0) t[0] *= 2.0;
            if (t[2] == 0) t[3] *= 2.0;
            if (t[3] == 0) t[2] *= 2.0;
            if (t[4] == 0) t[5] *= 2.0;
            if (t[5] == 0) t[4] *= 2.0;
        }
        for (int f = 0; f < 6; ++f) tt[(size_t)f * N + c] = t[f];
    }
}

// One step of the slopes (Glioma_MALAslopesRHS<3>, :152-182, then
// UpdateMALAslopes<3>, :215-223) from phi, sRho, sD before the step:
//   dsRho/dt = -ih2 Dw (sum tt) sRho_c + ih2 Dw sum tt_f sRho_f + phi (1 - phi)
//   dsD/dt   = -ih2 Dw (sum tt) sD_c + ih2 Dw sum tt_f sD_f
//              + ih2 sum tt_f phi_f - ih2 (sum tt) phi_c
// each sum and product in the reference's order, the rates rounded to Real,
// s += dt * rate in double.
template <typename Real>
__global__ void k_mala_slopes(int n, const Real *__restrict__ phi, const Real *__restrict__ sr,
                              const Real *__restrict__ sd, Real *__restrict__ sr_out, Real *__restrict__ sd_out,
                              const double *__restrict__ tt, Real Dw, double ih2, double dt) {
    const size_t N = (size_t)n * n * n;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
         c += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(c % n), y = (int)((c / n) % n), z = (int)(c / ((size_t)n * n));
        const size_t nn = (size_t)n, plane = nn * nn;
        const size_t nb[6] = {c - x + wrapm(x, n),
                              c - x + wrapp(x, n),
                              c + ((size_t)wrapm(y, n) - y) * nn,
                              c + ((size_t)wrapp(y, n) - y) * nn,
                              c + ((size_t)wrapm(z, n) - z) * plane,
                              c + ((size_t)wrapp(z, n) - z) * plane};
        double t[6], s[6], d[6], p[6];
        for (int f = 0; f < 6; ++f) {
            t[f] = tt[(size_t)f * N + c];
            s[f] = (double)sr[nb[f]];
            d[f] = (double)sd[nb[f]];
            p[f] = (double)phi[nb[f]];
        }
        const double s0 = (double)sr[c], d0 = (double)sd[c], p0 = (double)phi[c];
        const double tsum = t[0] + t[1] + t[2] + t[3] + t[4] + t[5];
        const double ihD = ih2 * (double)Dw;
        const double inR = ihD * (t[0] * s[0] + t[1] * s[1] + t[2] * s[2] + t[3] * s[3] + t[4] * s[4] + t[5] * s[5]);
        const double outR = -ih2 * (double)Dw * tsum * s0;
        const double reR = p0 * (1. - p0);
        const Real rr = (Real)(outR + inR + reR);
        const double inD = ihD * (t[0] * d[0] + t[1] * d[1] + t[2] * d[2] + t[3] * d[3] + t[4] * d[4] + t[5] * d[5]);
        const double outD = -ih2 * (double)Dw * tsum * d0;
        const double rin = ih2 * (t[0] * p[0] + t[1] * p[1] + t[2] * p[2] + t[3] * p[3] + t[4] * p[4] + t[5] * p[5]);
        const double rout = -ih2 * tsum * p0;
        const Real rd = (Real)(outD + inD + rin + rout);
        sr_out[c] = (Real)(s0 + dt * (double)rr);
        sd_out[c] = (Real)(d0 + dt * (double)rd);
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

int mala_steps(Handle &h, double Dw, double Dg, double rho, double dt, long nsteps) {
    // ratioD = Dg / Dw in Real, widened to double (Glioma_MALA_SlopesOperator.h:117)
    const double ratio = h.prec == GBG_PREC_F64 ? Dg / Dw : (double)((float)Dg / (float)Dw);
    const int g = grid_for(h);
    if (!h.mala_valid || h.mala_ratio != ratio) {
        if (h.prec == GBG_PREC_F64)
            k_mala_tables<double><<<g, 256, 0, h.stream>>>(h.n, h.pw, h.pg, ratio, h.mala_tt);
        else
            k_mala_tables<float><<<g, 256, 0, h.stream>>>(h.n, h.pw, h.pg, ratio, h.mala_tt);
        h.launches++;
        GBG_CUDA_TRY(cudaGetLastError());
        h.mala_ratio = ratio;
        h.mala_valid = true;
    }
    const double hh = 1.0 / h.n;
    const double ih2 = 1. / (hh * hh);
    for (long s = 0; s < nsteps; ++s) {
        const int c = h.cur;
        if (h.prec == GBG_PREC_F64) {
            k_mala_slopes<double><<<g, 256, 0, h.stream>>>(h.n, (const double *)h.phi[c], (const double *)h.sr[c],
                                                          (const double *)h.sd[c], (double *)h.sr[c ^ 1],
                                                          (double *)h.sd[c ^ 1], h.mala_tt, Dw, ih2, dt);
        } else {
            k_mala_slopes<float><<<g, 256, 0, h.stream>>>(h.n, (const float *)h.phi[c], (const float *)h.sr[c],
                                                         (const float *)h.sd[c], (float *)h.sr[c ^ 1],
                                                         (float *)h.sd[c ^ 1], h.mala_tt, (float)Dw, ih2, dt);
        }
        h.launches++;
        // the phi step reads the same phi[c] and toggles cur for phi and slopes
        if (int rc = exact_steps(h, Dw, Dg, rho, dt, 1)) return rc;
    }
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
}

}  // namespace gbg
