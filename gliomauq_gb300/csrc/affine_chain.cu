// The first stage of delayed-acceptance MCMC on the GPU: `steps` Metropolis
// steps on the screening density
//   log pi*(v) = log L(phi(v)) + log prior(v),
//   phi(v) = m * clamp(phi0 + sum_p c_p(v - u_ref) J_p, 0, 1)
// (the affine model of affine.cu, evaluated at the observation lists' cells
// from the same gathered columns) for B chains at once, one CTA per chain, so
// that a whole inner chain is one launch instead of one host round trip per
// step. The moves are those of the host sampler's inner chain
// (gliomauq_gb300/mcmc.py, da): with probability axis_prob a redraw of the
// symmetry coordinate from its prior conditional, accepted with the ratio of
// pi*'s likelihood factors; with probability ind_prob an independence
// proposal m + G xi for the other coordinates (a fixed Gaussian, accepted
// with the Metropolis-Hastings ratio of its density); otherwise a random
// walk v + step * C xi on the other coordinates. All three leave pi*
// invariant. Random numbers come from a
// counter-based hash (SplitMix64 finaliser, Steele, Lea & Flood 2014) of
// (seed, chain, step, draw), normals by the Box-Muller transform.
//
// Prior in the sampler's coordinates v: u = Ai v; theta_i = exp(u_i) where
// bit i of log_mask is set, else u_i; log prior = sum of those u_i (the
// log-Jacobian of the uniform prior on theta) inside the box lo <= theta <= hi
// with the seed voxel (rint of theta_2..4) inside the mask, -inf outside.
//
// Each observation point's model (phi0, the basis fields, the mask) and its
// observed values are one 16-float record (affine.cu builds them), read with
// four vector loads. The per-point likelihood terms are evaluated in float (this GPU's FP64 rate
// is a small fraction of its FP32 rate, and the screen only has to be one
// fixed function: the chain returns its own log pi* at the start and end
// points, which is what the second stage's ratio uses), summed in float per
// thread and in double across the block. The Bernoulli terms of
// HGG_Likelihood (:136-153) in a form without cancellation: with
// q = (u - uc)^2 / slope, alpha = 1 - e^-q / 2 above uc and e^-q / 2 below,
// so log alpha and log(1 - alpha) are log1p(-e^-q / 2) and log(1/2) - q.
#include <math_constants.h>

#include <cmath>

#include "gbg_internal.cuh"
#include "lik_terms.cuh"

namespace gbg {
namespace {

constexpr int kChainThreads = 512;
constexpr int kChainWarps = kChainThreads / 32;

struct ChainArgs {
    int steps, P, quad_axis, axis, log_mask, n;
    double axis_prob, step, ind_prob;
    double u_ref[6], chol[36], Ai[36], lo[6], hi[6], ulo[6], uhi[6];
    double ind_mean[6], ind_chol[36], ind_inv[36];
    const unsigned char *mask;
    unsigned long long seed;
    const float4 *rec;  // per observation point, PET list then T1/T2 list: 16 floats
    int n_pet, n_ti;
    double pet_scale, t1_uc, t2_uc, is2, pet_sigma2;
    double *v, *lp_start, *lp_end;
    int *counts;
};

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// uniform in (0, 1] from (seed, chain, step, draw)
__device__ __forceinline__ double uniform01(unsigned long long seed, int chain, int step, int k) {
    unsigned long long x = mix64(seed ^ mix64((unsigned long long)chain));
    x = mix64(x ^ ((unsigned long long)step << 8 | (unsigned long long)k));
    return (double)((x >> 11) + 1) * (1.0 / 9007199254740992.0);
}

__device__ double prior_logp(const ChainArgs &a, const double *v) {
    double u[6], th[6], jac = 0.0;
    for (int i = 0; i < 6; ++i) {
        double s = 0.0;
        for (int j = 0; j < 6; ++j) s += a.Ai[i * 6 + j] * v[j];
        u[i] = s;
    }
    for (int i = 0; i < 6; ++i) {
        if ((a.log_mask >> i) & 1) {
            th[i] = exp(u[i]);
            jac += u[i];
        } else {
            th[i] = u[i];
        }
    }
    for (int i = 0; i < 6; ++i)
        if (!(th[i] >= a.lo[i] && th[i] <= a.hi[i])) return -CUDART_INF;
    int c[3];
    for (int k = 0; k < 3; ++k) {
        const double r = rint(th[2 + k]);
        if (!(r >= 0.0 && r < (double)a.n)) return -CUDART_INF;
        c[k] = (int)r;
    }
    if (!a.mask[((size_t)c[2] * a.n + c[1]) * a.n + c[0]]) return -CUDART_INF;
    return jac;
}

// coordinate `axis` of v redrawn from the prior conditional given the others:
// on the line v + t e_axis the prior density is exp(alpha t) on the interval
// the box allows; v is left unchanged when the line misses the box
__device__ void redraw_axis(const ChainArgs &a, double *v, double q) {
    const int ax = a.axis;
    double u[6];
    for (int i = 0; i < 6; ++i) {
        double s = 0.0;
        for (int j = 0; j < 6; ++j) s += a.Ai[i * 6 + j] * v[j];
        u[i] = s;
    }
    double t_lo = -CUDART_INF, t_hi = CUDART_INF, alpha = 0.0;
    for (int i = 0; i < 6; ++i) {
        if (!((a.log_mask >> i) & 1)) continue;
        const double col = a.Ai[i * 6 + ax];
        alpha += col;
        if (col == 0.0) continue;
        const double b1 = (a.ulo[i] - u[i]) / col, b2 = (a.uhi[i] - u[i]) / col;
        t_lo = fmax(t_lo, fmin(b1, b2));
        t_hi = fmin(t_hi, fmax(b1, b2));
    }
    if (!(isfinite(t_lo) && isfinite(t_hi) && t_hi > t_lo)) return;
    double t;
    if (fabs(alpha) < 1e-12)
        t = t_lo + q * (t_hi - t_lo);
    else
        t = t_lo + log1p(q * expm1(alpha * (t_hi - t_lo))) / alpha;
    v[ax] += t;
}

__device__ void coefficients(const ChainArgs &a, const double *v, double *c) {
    double d[6];
    for (int i = 0; i < 6; ++i) d[i] = v[i] - a.u_ref[i];
    for (int i = 0; i < 6; ++i) c[i] = d[i];
    if (a.quad_axis >= 0) {
        const int ax = a.quad_axis;
        c[6] = 0.5 * (d[ax] * d[ax]);
        int k = 7;
        for (int i = 0; i < 6; ++i)
            if (i != ax) c[k++] = d[ax] * d[i];
    }
}

// log Bernoulli(alpha(u)) of observation y in float, without cancellation
__device__ __forceinline__ float log_bernoulli_f(float u, float y, float uc, float is2) {
    const float d = u - uc;
    const float q = d * d * is2;
    const float lhalf_q = -0.69314718f - q;          // log(e^-q / 2)
    const float l1m = log1pf(-0.5f * expf(-q));      // log(1 - e^-q / 2)
    float la, lna;                                   // log alpha, log(1 - alpha)
    if (d > 0.f) {
        la = l1m;
        lna = lhalf_q;
    } else if (d < 0.f) {
        la = lhalf_q;
        lna = l1m;
    } else {
        la = lna = -0.69314718f;
    }
    return y == 1.f ? la : lna;
}

// log L of the model with coefficients s_c (block-wide; the total on thread 0).
// Point i (PET list first, then the T1/T2 list) is one 16-float record:
// phi0, J_0 .. J_{P-1}, mask, then PET or T1, T2.
template <int P>
__device__ double eval_lik(const ChainArgs &a, const double *s_c, double (*s_red)[kChainWarps]) {
    float cf[P];
#pragma unroll
    for (int p = 0; p < P; ++p) cf[p] = (float)s_c[p];
    const float scale = (float)a.pet_scale, uc1 = (float)a.t1_uc, uc2 = (float)a.t2_uc, is2 = (float)a.is2;
    float fp = 0.f, f1 = 0.f, f2 = 0.f;
    const int items = a.n_pet + a.n_ti;
#pragma unroll 2
    for (int i = threadIdx.x; i < items; i += kChainThreads) {
        float x[16];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float4 v = __ldg(a.rec + (size_t)i * 4 + q);
            x[4 * q] = v.x;
            x[4 * q + 1] = v.y;
            x[4 * q + 2] = v.z;
            x[4 * q + 3] = v.w;
        }
        float u = x[0];
#pragma unroll
        for (int p = 0; p < P; ++p) u = fmaf(cf[p], x[1 + p], u);
        u = fminf(fmaxf(u, 0.f), 1.f);
        if (x[P + 1] == 0.f) u = 0.f;
        if (i < a.n_pet) {
            const float r = u - scale * x[P + 2];
            fp += r * r;
        } else {
            f1 += log_bernoulli_f(u, x[P + 2], uc1, is2);
            f2 += log_bernoulli_f(u, x[P + 3], uc2, is2);
        }
    }
    double sp = warp_sum((double)fp), s1 = warp_sum((double)f1), s2 = warp_sum((double)f2);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        s_red[0][w] = sp;
        s_red[1][w] = s1;
        s_red[2][w] = s2;
    }
    __syncthreads();
    double total = 0.0;
    if (threadIdx.x == 0) {
        double t[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < 3; ++k)
            for (int j = 0; j < kChainWarps; ++j) t[k] += s_red[k][j];
        const double p1 = -0.5 * a.n_pet * log(2. * 3.14159265358979323846 * a.pet_sigma2);
        const double p2 = -0.5 * (1. / a.pet_sigma2) * t[0];
        total = (p1 + p2) + t[1] + t[2];
    }
    __syncthreads();
    return total;
}

template <int P>
__global__ void __launch_bounds__(kChainThreads) k_affine_chain(ChainArgs a) {
    const int b = blockIdx.x;
    __shared__ double s_c[16];
    __shared__ double s_red[3][kChainWarps];
    __shared__ int s_eval;
    double v[6], y[6], lpv = 0.0, lpy = 0.0, ly = 0.0;
    int cnt[6] = {0, 0, 0, 0, 0, 0};
    bool jump = false, indep = false;
    double lqd = 0.0;  // log proposal-density ratio of an independence move
    if (threadIdx.x == 0) {
        for (int i = 0; i < 6; ++i) v[i] = a.v[(size_t)b * 6 + i];
        lpv = prior_logp(a, v);
        coefficients(a, v, s_c);
        s_eval = isfinite(lpv) ? 1 : 0;
    }
    __syncthreads();
    {
        const double L = s_eval ? eval_lik<P>(a, s_c, s_red) : 0.0;
        if (threadIdx.x == 0) {
            ly = s_eval ? L + lpv : -CUDART_INF;
            a.lp_start[b] = ly;
        }
    }
    __syncthreads();  // every thread has read s_eval before thread 0 rewrites it
    for (int s = 0; s < a.steps; ++s) {
        if (threadIdx.x == 0) {
            const double um = uniform01(a.seed, b, s, 0);
            jump = a.axis >= 0 && um <= a.axis_prob;
            indep = !jump && um <= (a.axis >= 0 ? a.axis_prob : 0.0) + a.ind_prob;
            for (int i = 0; i < 6; ++i) y[i] = v[i];
            if (jump) {
                redraw_axis(a, y, uniform01(a.seed, b, s, 1));
            } else if (indep) {
                // y = m + G xi on the coordinates other than the axis; the
                // density ratio q(v) / q(y) with z = G^-1 (x - m)
                double xi[6], zv[6];
                for (int k = 0; k < 3; ++k) {
                    const float r = sqrtf(-2.0f * logf((float)uniform01(a.seed, b, s, 2 + 2 * k)));
                    float sn, cs;
                    sincospif(2.0f * (float)uniform01(a.seed, b, s, 3 + 2 * k), &sn, &cs);
                    xi[2 * k] = (double)(r * cs);
                    xi[2 * k + 1] = (double)(r * sn);
                }
                if (a.axis >= 0) xi[a.axis] = 0.0;
                double qy = 0.0, qv = 0.0;
                for (int i = 0; i < 6; ++i) {
                    if (i == a.axis) continue;
                    double d = 0.0, z = 0.0;
                    for (int j = 0; j < 6; ++j) {
                        d += a.ind_chol[i * 6 + j] * xi[j];
                        z += a.ind_inv[i * 6 + j] * (v[j] - a.ind_mean[j]);
                    }
                    y[i] = a.ind_mean[i] + d;
                    zv[i] = z;
                    qy += xi[i] * xi[i];
                    qv += zv[i] * zv[i];
                }
                lqd = 0.5 * (qy - qv);  // log q(v) - log q(y)
            } else {
                // normals in float: their precision does not matter, the
                // state they move stays double
                double xi[6];
                for (int k = 0; k < 3; ++k) {
                    const float r = sqrtf(-2.0f * logf((float)uniform01(a.seed, b, s, 2 + 2 * k)));
                    float sn, cs;
                    sincospif(2.0f * (float)uniform01(a.seed, b, s, 3 + 2 * k), &sn, &cs);
                    xi[2 * k] = (double)(r * cs);
                    xi[2 * k + 1] = (double)(r * sn);
                }
                for (int i = 0; i < 6; ++i) {
                    double d = 0.0;
                    for (int j = 0; j < 6; ++j) d += a.chol[i * 6 + j] * xi[j];
                    y[i] = v[i] + a.step * d;
                }
                if (a.axis >= 0) y[a.axis] = v[a.axis];
            }
            lpy = prior_logp(a, y);
            coefficients(a, y, s_c);
            s_eval = isfinite(lpy) ? 1 : 0;
        }
        __syncthreads();
        const double L = s_eval ? eval_lik<P>(a, s_c, s_red) : 0.0;
        if (threadIdx.x == 0) {
            const double lq = s_eval ? L + lpy : -CUDART_INF;
            // a prior-conditional redraw: its proposal density cancels the
            // prior; an independence move: the proposal density ratio
            const double corr = jump ? lpv - lpy : (indep ? lqd : 0.0);
            const double logu = log(uniform01(a.seed, b, s, 8));
            const bool acc = isfinite(lq) && (logu < lq - ly + corr);
            if (acc) {
                for (int i = 0; i < 6; ++i) v[i] = y[i];
                ly = lq;
                lpv = lpy;
            }
            const int kind = jump ? 2 : (indep ? 4 : 0);
            cnt[kind] += acc ? 1 : 0;
            cnt[kind + 1] += 1;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < 6; ++i) a.v[(size_t)b * 6 + i] = v[i];
        a.lp_end[b] = ly;
        for (int k = 0; k < 6; ++k) a.counts[(size_t)b * 6 + k] = cnt[k];
    }
}

}  // namespace

int affine_set_prior_mask(Handle &h, const unsigned char *mask) {
    if (!h.aff_mask) GBG_CUDA_TRY(cudaMalloc((void **)&h.aff_mask, h.N));
    GBG_CUDA_TRY(cudaMemcpyAsync(h.aff_mask, mask, h.N, cudaMemcpyHostToDevice, h.stream));
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    return GBG_OK;
}

int affine_chain(Handle &h, const gbg_affine_chain_opts &o, int B, int steps, unsigned long long seed,
                 double *v, double *lp_start, double *lp_end, int *counts) {
    const int P = o.quad_axis >= 0 ? 12 : 6;
    if (!h.aff_J || h.aff_P != P) {
        set_error("affine chain: the affine model must have 6 (no quad_axis) or 12 basis fields");
        return GBG_ERR_STATE;
    }
    if (!h.aff_mask) {
        set_error("affine chain: prior mask not set");
        return GBG_ERR_STATE;
    }
    if (!h.obs.valid) {
        set_error("observations not set");
        return GBG_ERR_STATE;
    }
    if (h.aff_cols_stale)
        if (int rc = affine_gather_columns(h)) return rc;
    // device scratch: v (B x 6), lp_start, lp_end (B), counts (B x 4)
    const size_t need = (size_t)B * (8 * sizeof(double) + 6 * sizeof(int));
    if (need > h.aff_chain_bytes) {
        if (h.aff_chain) cudaFree(h.aff_chain);
        h.aff_chain = nullptr;
        h.aff_chain_bytes = 0;
        GBG_CUDA_TRY(cudaMalloc(&h.aff_chain, need));
        h.aff_chain_bytes = need;
    }
    double *d_v = (double *)h.aff_chain, *d_l0 = d_v + (size_t)B * 6, *d_l1 = d_l0 + B;
    int *d_cnt = (int *)(d_l1 + B);
    ChainArgs a;
    a.steps = steps;
    a.P = P;
    a.quad_axis = o.quad_axis;
    a.axis = o.axis;
    a.log_mask = o.log_mask;
    a.n = h.n;
    a.axis_prob = o.axis_prob;
    a.ind_prob = o.ind_prob;
    for (int i = 0; i < 6; ++i) a.ind_mean[i] = o.ind_mean[i];
    for (int i = 0; i < 36; ++i) {
        a.ind_chol[i] = o.ind_chol[i];
        a.ind_inv[i] = o.ind_inv[i];
    }
    a.step = o.step;
    for (int i = 0; i < 6; ++i) {
        a.u_ref[i] = o.u_ref[i];
        a.lo[i] = o.lo[i];
        a.hi[i] = o.hi[i];
        const bool lg = (o.log_mask >> i) & 1;
        a.ulo[i] = lg ? std::log(o.lo[i]) : o.lo[i];
        a.uhi[i] = lg ? std::log(o.hi[i]) : o.hi[i];
    }
    for (int i = 0; i < 36; ++i) {
        a.chol[i] = o.chol[i];
        a.Ai[i] = o.Ai[i];
    }
    a.mask = h.aff_mask;
    a.seed = seed;
    a.rec = h.aff_rec;
    a.n_pet = h.obs.n_pet;
    a.n_ti = h.obs.n_ti;
    a.pet_scale = h.obs.pet_scale;
    a.t1_uc = h.obs.t1_uc;
    a.t2_uc = h.obs.t2_uc;
    a.is2 = 1. / h.obs.slope;
    a.pet_sigma2 = h.obs.pet_sigma2;
    a.v = d_v;
    a.lp_start = d_l0;
    a.lp_end = d_l1;
    a.counts = d_cnt;
    GBG_CUDA_TRY(cudaMemcpyAsync(d_v, v, (size_t)B * 6 * sizeof(double), cudaMemcpyHostToDevice, h.stream));
    if (P == 12)
        k_affine_chain<12><<<B, kChainThreads, 0, h.stream>>>(a);
    else
        k_affine_chain<6><<<B, kChainThreads, 0, h.stream>>>(a);
    h.launches++;
    GBG_CUDA_TRY(cudaGetLastError());
    GBG_CUDA_TRY(cudaMemcpyAsync(v, d_v, (size_t)B * 6 * sizeof(double), cudaMemcpyDeviceToHost, h.stream));
    GBG_CUDA_TRY(cudaMemcpyAsync(lp_start, d_l0, (size_t)B * sizeof(double), cudaMemcpyDeviceToHost, h.stream));
    GBG_CUDA_TRY(cudaMemcpyAsync(lp_end, d_l1, (size_t)B * sizeof(double), cudaMemcpyDeviceToHost, h.stream));
    if (counts)
        GBG_CUDA_TRY(cudaMemcpyAsync(counts, d_cnt, (size_t)B * 6 * sizeof(int), cudaMemcpyDeviceToHost, h.stream));
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    return GBG_OK;
}

}  // namespace gbg
