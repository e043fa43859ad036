// Affine density model for cheap screening around a posterior mode:
//   phi_s = m * clamp(phi0 + sum_p delta_{s,p} J_p, 0, 1)
// phi0 is the final density at a reference sample, J_p basis fields (the
// derivatives along the sampler's coordinates, and optionally second-order
// terms whose coefficients the caller forms, such as delta_0^2 / 2), m the
// fast path's tissue mask. The likelihood reads the density only at its
// observation lists' cells, so phi0, J and m are gathered once at those cells
// (k_affine_gather, when the model or the observations change) and each
// evaluation forms the B models' densities there inside the likelihood
// reduction: per model (P + 2) floats per observation instead of a whole
// n^3 field written and read back.
#include <algorithm>

#include "gbg_internal.cuh"

namespace gbg {
namespace {

constexpr int kAffineMaxP = 16;

// cols block of one list: row 0 phi0, rows 1..P the basis fields, row P+1 the
// mask, each `len` floats, at the list's cells idx[0..len)
__global__ void k_affine_gather(int len, const int *__restrict__ idx, size_t N, int P,
                                const float *__restrict__ phi0, const float *__restrict__ J,
                                const float *__restrict__ msk, float *__restrict__ cols) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
        const size_t c = (size_t)idx[i];
        cols[i] = phi0[c];
        for (int p = 0; p < P; ++p) cols[(size_t)(1 + p) * len + i] = J[(size_t)p * N + c];
        cols[(size_t)(P + 1) * len + i] = msk[c];
    }
}

// one 16-float record per observation point for the screening chain: phi0,
// the P basis fields, the mask, then the observation values (PET; or T1, T2),
// zero padding
__global__ void k_affine_records(int len, int P, const float *__restrict__ cols, const double *__restrict__ v1,
                                 const double *__restrict__ v2, float4 *__restrict__ rec) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
        float r[16];
        for (int k = 0; k < 16; ++k) r[k] = 0.f;
        for (int k = 0; k < P + 2; ++k) r[k] = cols[(size_t)k * len + i];
        r[P + 2] = (float)v1[i];
        if (v2) r[P + 3] = (float)v2[i];
        for (int q = 0; q < 4; ++q) rec[(size_t)i * 4 + q] = make_float4(r[4 * q], r[4 * q + 1], r[4 * q + 2], r[4 * q + 3]);
    }
}

}  // namespace

int affine_gather_columns(Handle &h) {
    const int P = h.aff_P;
    const size_t need = (size_t)(P + 2) * ((size_t)h.obs.n_pet + (size_t)h.obs.n_ti);
    if (need > h.aff_cols_cap) {
        if (h.aff_cols) cudaFree(h.aff_cols);
        h.aff_cols = nullptr;
        h.aff_cols_cap = 0;
        GBG_CUDA_TRY(cudaMalloc((void **)&h.aff_cols, need * sizeof(float)));
        h.aff_cols_cap = need;
    }
    const int lens[2] = {h.obs.n_pet, h.obs.n_ti};
    const int *idx[2] = {h.obs.pet_idx, h.obs.ti_idx};
    float *dst = h.aff_cols;
    for (int l = 0; l < 2; ++l) {
        if (lens[l] > 0) {
            const int blocks = (lens[l] + 255) / 256;
            k_affine_gather<<<blocks < h.num_sms * 8 ? blocks : h.num_sms * 8, 256, 0, h.stream>>>(
                lens[l], idx[l], h.N, P, h.aff_phi0, h.aff_J, h.msk, dst);
            h.launches++;
        }
        dst += (size_t)(P + 2) * lens[l];
    }
    // per-point records for the screening chain (P + 4 <= 16 floats)
    const size_t npts = (size_t)h.obs.n_pet + (size_t)h.obs.n_ti;
    if (P + 4 <= 16) {
        if (npts > h.aff_rec_cap) {
            if (h.aff_rec) cudaFree(h.aff_rec);
            h.aff_rec = nullptr;
            h.aff_rec_cap = 0;
            GBG_CUDA_TRY(cudaMalloc((void **)&h.aff_rec, (npts ? npts : 1) * 4 * sizeof(float4)));
            h.aff_rec_cap = npts ? npts : 1;
        }
        if (h.obs.n_pet > 0)
            k_affine_records<<<std::min((h.obs.n_pet + 255) / 256, h.num_sms * 8), 256, 0, h.stream>>>(
                h.obs.n_pet, P, h.aff_cols, h.obs.pet_val, nullptr, h.aff_rec);
        if (h.obs.n_ti > 0)
            k_affine_records<<<std::min((h.obs.n_ti + 255) / 256, h.num_sms * 8), 256, 0, h.stream>>>(
                h.obs.n_ti, P, h.aff_cols + (size_t)(P + 2) * h.obs.n_pet, h.obs.t1_val, h.obs.t2_val,
                h.aff_rec + (size_t)h.obs.n_pet * 4);
        h.launches += 2;
    }
    GBG_CUDA_TRY(cudaGetLastError());
    h.aff_cols_stale = false;
    return GBG_OK;
}

int affine_set(Handle &h, int P, const float *phi0, const float *J) {
    if (P < 1 || P > kAffineMaxP) {
        set_error("affine model: 1 <= P <= 16 basis fields");
        return GBG_ERR_ARG;
    }
    if (int rc = fast_build_tables(h, (double)0.1f)) return rc;
    if (!h.aff_phi0) GBG_CUDA_TRY(cudaMalloc((void **)&h.aff_phi0, h.N * sizeof(float)));
    if (h.aff_P < P) {
        if (h.aff_J) cudaFree(h.aff_J);
        h.aff_J = nullptr;
        h.aff_P = 0;
        GBG_CUDA_TRY(cudaMalloc((void **)&h.aff_J, (size_t)P * h.N * sizeof(float)));
    }
    h.aff_P = P;
    GBG_CUDA_TRY(cudaMemcpyAsync(h.aff_phi0, phi0, h.N * sizeof(float), cudaMemcpyHostToDevice, h.stream));
    GBG_CUDA_TRY(cudaMemcpyAsync(h.aff_J, J, (size_t)P * h.N * sizeof(float), cudaMemcpyHostToDevice, h.stream));
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    h.aff_cols_stale = true;
    return GBG_OK;
}

int affine_loglik(Handle &h, int B, const double *delta_host, gbg_lik_result *lik_device) {
    if (!h.aff_J || h.aff_P < 1) {
        set_error("affine model not set");
        return GBG_ERR_STATE;
    }
    if (!h.obs.valid) {
        set_error("observations not set");
        return GBG_ERR_STATE;
    }
    const int P = h.aff_P;
    if ((size_t)B * P > h.aff_delta_cap) {
        if (h.aff_delta) cudaFree(h.aff_delta);
        h.aff_delta = nullptr;
        h.aff_delta_cap = 0;
        GBG_CUDA_TRY(cudaMalloc((void **)&h.aff_delta, (size_t)B * P * sizeof(double)));
        h.aff_delta_cap = (size_t)B * P;
    }
    if (h.aff_cols_stale)
        if (int rc = affine_gather_columns(h)) return rc;
    GBG_CUDA_TRY(cudaMemcpyAsync(h.aff_delta, delta_host, (size_t)B * P * sizeof(double), cudaMemcpyHostToDevice,
                                 h.stream));
    return lik_evaluate_affine(h, h.aff_cols, P, h.aff_delta, B, lik_device);
}

}  // namespace gbg
