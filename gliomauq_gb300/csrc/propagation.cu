// Posterior propagation statistics: per-cell mean and variance of S density
// fields, as the reference's propagation tool computes them over the
// samples' HGG_data.dat files (Glioma_HG_Propagation::_ic_PatientCasePropagation,
// source/Glioma/Glioma_HG_Propagation.cpp:346-440, then PropagationStatistics,
// Glioma_PropagationStatisticsOperator.h:24-50), in its default Real = float:
//   m = sum_s u_s                      (float, samples in order)
//   v = sum_s (u_s - m / S')^2         (float; m / S' = (1/S as float) * m)
//   mean = m * (1/S), var = v * (1/S)  (float)
// where a field value enters as the double it was written as, so each sum
// step is a double operation rounded to float. With reference_rules, cells
// with a zero x, y or z index keep mean = var = 0: the tool accumulates only
// mapped indices in (0, size] (:380-384, :432).
//
// One thread per cell, the S fields read in sample order (coalesced along the
// cells), twice: the second pass needs the finished sum. Compiled with
// -fmad=false: every product and sum rounds on its own.
#include "gbg_internal.cuh"

namespace gbg {
namespace {

struct FieldSource {
    const float *f0, *f1;     // fields of sample s at s * N in f0, or in f1 when
    const SampleRec *recs;    // recs is non-null and recs[s].nsteps is odd
    __device__ __forceinline__ const float *field(int s, size_t N) const {
        const float *b = (recs && (recs[s].nsteps & 1)) ? f1 : f0;
        return b + (size_t)s * N;
    }
};

__global__ void k_field_stats(int n, int S, FieldSource src, int reference_rules, float *__restrict__ mean,
                              float *__restrict__ var) {
    const size_t N = (size_t)n * n * n;
    const float inv = (float)(1. / S);
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N; c += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(c % n), y = (int)((c / n) % n), z = (int)(c / ((size_t)n * n));
        if (reference_rules && (x == 0 || y == 0 || z == 0)) {
            mean[c] = 0.0f;
            var[c] = 0.0f;
            continue;
        }
        float m = 0.0f;
        for (int s = 0; s < S; ++s) m = (float)((double)m + (double)src.field(s, N)[c]);
        const float p = __fmul_rn(inv, m);
        float v = 0.0f;
        for (int s = 0; s < S; ++s) {
            const float t = (float)((double)src.field(s, N)[c] - (double)p);
            v = __fadd_rn(v, __fmul_rn(t, t));
        }
        mean[c] = __fmul_rn(m, inv);
        var[c] = __fmul_rn(v, inv);
    }
}

int launch_stats(int num_sms, cudaStream_t st, int n, int S, const FieldSource &src, int reference_rules,
                 float *mean, float *var) {
    const size_t N = (size_t)n * n * n;
    size_t blocks = (N + 255) / 256;
    const size_t cap = (size_t)(num_sms > 0 ? num_sms : 132) * 8;
    if (blocks > cap) blocks = cap;
    k_field_stats<<<(unsigned)blocks, 256, 0, st>>>(n, S, src, reference_rules, mean, var);
    GBG_CUDA_TRY(cudaGetLastError());
    return GBG_OK;
}

}  // namespace

int batch_statistics(Handle &h, const gbg_sample *samples_device, int S, const gbg_batch_opts &o,
                     int reference_rules, float *mean_device, float *var_device) {
    if (int rc = batch_solve_device(h, samples_device, S, o, nullptr, nullptr)) return rc;
    FieldSource src{h.bphi[0], h.bphi[1], batch_unsorted(h)};
    h.launches++;
    return launch_stats(h.num_sms, h.stream, h.n, S, src, reference_rules, mean_device, var_device);
}

}  // namespace gbg

extern "C" int gbg_field_statistics(int n, const float *fields_device, int S, int reference_rules,
                                    float *mean_device, float *var_device, void *stream) {
    if (n < 1 || n > 1024 || S < 1 || !fields_device || !mean_device || !var_device) {
        gbg::set_error("gbg_field_statistics: bad argument");
        return GBG_ERR_ARG;
    }
    int dev = 0, sms = 0;
    GBG_CUDA_TRY(cudaGetDevice(&dev));
    GBG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    gbg::FieldSource src{fields_device, fields_device, nullptr};
    return gbg::launch_stats(sms, static_cast<cudaStream_t>(stream), n, S, src, reference_rules, mean_device,
                             var_device);
}
