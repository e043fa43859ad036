// Affine density model for cheap screening around a posterior mode:
//   phi_s = m * clamp(phi0 + sum_p delta_{s,p} J_p, 0, 1)
// phi0 is the final density at a reference sample, J_p basis fields (the
// derivatives along the sampler's coordinates, and optionally second-order
// terms whose coefficients the caller forms, such as delta_0^2 / 2), m the
// fast path's tissue mask. B such fields are formed in one pass over phi0
// and J (a thread owns one cell and writes it for every model; phi0 and J
// are read once per launch) and go through the handle's likelihood kernel.
#include "gbg_internal.cuh"

namespace gbg {
namespace {

constexpr int kAffineMaxP = 16;

__global__ void k_affine_fields(size_t N, int B, int P, const float *__restrict__ phi0,
                                const float *__restrict__ J, const double *__restrict__ delta,
                                const float *__restrict__ msk, float *__restrict__ out) {
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N; c += (size_t)gridDim.x * blockDim.x) {
        const float base = phi0[c];
        float jc[kAffineMaxP];
#pragma unroll
        for (int p = 0; p < kAffineMaxP; ++p) jc[p] = p < P ? J[(size_t)p * N + c] : 0.f;
        const bool tissue = msk[c] != 0.f;
        for (int s = 0; s < B; ++s) {
            float v = base;
#pragma unroll
            for (int p = 0; p < kAffineMaxP; ++p)
                if (p < P) v = fmaf((float)delta[(size_t)s * P + p], jc[p], v);
            v = fminf(fmaxf(v, 0.f), 1.f);
            out[(size_t)s * N + c] = tissue ? v : 0.f;
        }
    }
}

}  // namespace

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
    return GBG_OK;
}

int affine_loglik(Handle &h, int B, const double *delta_host, gbg_lik_result *lik_device) {
    if (!h.aff_J || h.aff_P < 1) {
        set_error("affine model not set");
        return GBG_ERR_STATE;
    }
    const int P = h.aff_P;
    if ((size_t)B > h.aff_out_cap) {
        if (h.aff_out) cudaFree(h.aff_out);
        h.aff_out = nullptr;
        h.aff_out_cap = 0;
        GBG_CUDA_TRY(cudaMalloc((void **)&h.aff_out, (size_t)B * h.N * sizeof(float)));
        h.aff_out_cap = B;
    }
    if ((size_t)B * P > h.aff_delta_cap) {
        if (h.aff_delta) cudaFree(h.aff_delta);
        h.aff_delta = nullptr;
        h.aff_delta_cap = 0;
        GBG_CUDA_TRY(cudaMalloc((void **)&h.aff_delta, (size_t)B * P * sizeof(double)));
        h.aff_delta_cap = (size_t)B * P;
    }
    GBG_CUDA_TRY(cudaMemcpyAsync(h.aff_delta, delta_host, (size_t)B * P * sizeof(double), cudaMemcpyHostToDevice,
                                 h.stream));
    const size_t blocks = (h.N + 255) / 256, cap = (size_t)h.num_sms * 8;
    k_affine_fields<<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, h.stream>>>(h.N, B, P, h.aff_phi0, h.aff_J,
                                                                                   h.aff_delta, h.msk, h.aff_out);
    h.launches++;
    GBG_CUDA_TRY(cudaGetLastError());
    return lik_evaluate(h, h.aff_out, nullptr, B, lik_device);
}

}  // namespace gbg
