// The C ABI of libgbglioma (include/gbglioma.h): handle lifetime, state
// upload/download, and the entry points that replace the reference's block
// processing of the RD step, its time loop and its likelihood.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "gbg_internal.cuh"

namespace gbg {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

// Glioma_HG_UQ::run, source/Glioma/Glioma_HG_UQ.cpp:519-539. In the float
// build Dw, Dg and rho are Real = float: Dw is read as float, Dw/(L*L) is a
// double division rounded back to float, Dg = 0.1*Dw likewise.
void reference_dt(int n, double Dw_file, double L, bool f32, double *dt, double *Dw, double *Dg,
                  double *rho) {
    double dw, dg;
    if (f32) {
        const float dwf = (float)((double)(float)Dw_file / (L * L));
        const float dgf = (float)(0.1 * (double)dwf);
        dw = dwf;
        dg = dgf;
        *rho = (double)(float)*rho;
    } else {
        dw = Dw_file / (L * L);
        dg = 0.1 * dw;
    }
    const double h = 1. / n;
    const double mx = dw >= dg ? dw : dg;
    *dt = 0.99 * h * h / (2. * 3 * mx);
    *Dw = dw;
    *Dg = dg;
}

long reference_num_steps(double dt, double tend) {
    double t = 0.0;
    long k = 0;
    while (t <= tend && k < 100000000L) {
        t += dt;
        ++k;
    }
    return k;
}

}  // namespace gbg

using gbg::Handle;
using gbg::set_error;

namespace {

int check_handle(gbg_handle *hh) {
    if (!hh) {
        set_error("null handle");
        return GBG_ERR_ARG;
    }
    return GBG_OK;
}

size_t storage_bytes(int prec) { return prec == GBG_PREC_F64 ? sizeof(double) : sizeof(float); }

bool all_finite(const double *a, size_t n) {
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(a[i])) return false;
    return true;
}

void free_handle(Handle &h) {
    void *ptrs[] = {h.pw, h.pg, h.phi[0], h.phi[1], h.b0, h.dfx, h.dfy, h.dfz, h.cx, h.cy, h.cz,
                    h.msk, h.cxs, h.sr[0], h.sr[1], h.sd[0], h.sd[1], h.mala_tt, h.bphi[0], h.bphi[1], h.bwork, h.dev_status, h.barrier,
                    h.obs.pet_idx, h.obs.pet_val, h.obs.ti_idx, h.obs.t1_val, h.obs.t2_val,
                    h.lik_partials, h.lik_out, h.adj_ws, h.aff_phi0, h.aff_J, h.aff_cols, h.aff_delta, h.aff_mask, h.aff_chain, h.aff_rec,
                    h.tile_live, h.live_list, h.live_count};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (cudaEvent_t e : h.ev_pop)
        if (e) cudaEventDestroy(e);
    gbg::batch_graphs_clear(h);
    if (h.is_amr) gbg::amr_free(h);
    if (h.stream) cudaStreamDestroy(h.stream);
}

int ensure_lik_out(Handle &h, int S) {
    if (h.lik_out_cap >= S) return GBG_OK;
    ++h.state_gen;
    if (h.lik_out) cudaFree(h.lik_out);
    h.lik_out = nullptr;
    h.lik_out_cap = 0;
    GBG_CUDA_TRY(cudaMalloc(&h.lik_out, sizeof(gbg_lik_result) * (size_t)S));
    h.lik_out_cap = S;
    return GBG_OK;
}

}  // namespace

extern "C" {

const char *gbg_last_error(void) { return gbg::g_last_error.c_str(); }

int gbg_version(int *major, int *minor) {
    if (major) *major = GBG_VERSION_MAJOR;
    if (minor) *minor = GBG_VERSION_MINOR;
    return GBG_OK;
}

int gbg_create(const gbg_config *cfg, gbg_handle **out) {
    if (!cfg || !out) {
        set_error("null argument");
        return GBG_ERR_ARG;
    }
    *out = nullptr;
    if (cfg->n < 4 || cfg->n > 1024 || cfg->precision < GBG_PREC_F64 ||
        cfg->precision > GBG_PREC_F32 || cfg->max_samples < 0) {
        set_error("bad configuration");
        return GBG_ERR_ARG;
    }
    int ndev = 0;
    GBG_CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (cfg->device < 0 || cfg->device >= ndev) {
        set_error("device ordinal out of range");
        return GBG_ERR_ARG;
    }
    GBG_CUDA_TRY(cudaSetDevice(cfg->device));
    gbg_handle *hh = new gbg_handle();
    Handle &h = hh->h;
    h.n = cfg->n;
    h.N = (size_t)cfg->n * cfg->n * cfg->n;
    h.prec = cfg->precision;
    h.device = cfg->device;
    h.max_samples = cfg->max_samples;
    auto fail = [&](int rc) {
        free_handle(h);
        delete hh;
        return rc;
    };
#define TRY_ALLOC(ptr, bytes)                                                  \
    do {                                                                       \
        cudaError_t e = cudaMalloc((void **)&(ptr), (bytes));                  \
        if (e != cudaSuccess) {                                                \
            set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));    \
            return fail(e == cudaErrorMemoryAllocation ? GBG_ERR_NOMEM : GBG_ERR_CUDA); \
        }                                                                      \
    } while (0)
    if (cudaDeviceGetAttribute(&h.num_sms, cudaDevAttrMultiProcessorCount, h.device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&h.ev_pop[0]) != cudaSuccess || cudaEventCreate(&h.ev_pop[1]) != cudaSuccess) {
        set_error("stream creation failed");
        return fail(GBG_ERR_CUDA);
    }
    const size_t sb = storage_bytes(h.prec);
    TRY_ALLOC(h.pw, h.N * sizeof(double));
    TRY_ALLOC(h.pg, h.N * sizeof(double));
    TRY_ALLOC(h.phi[0], h.N * sb);
    TRY_ALLOC(h.phi[1], h.N * sb);
    if (h.prec == GBG_PREC_F32) {
        TRY_ALLOC(h.cx, h.N * sizeof(float));
        TRY_ALLOC(h.cy, h.N * sizeof(float));
        TRY_ALLOC(h.cz, h.N * sizeof(float));
        TRY_ALLOC(h.msk, h.N * sizeof(float));
        TRY_ALLOC(h.cxs, h.N * sizeof(float));
        if (h.max_samples > 0) {
            TRY_ALLOC(h.bphi[0], h.N * (size_t)h.max_samples * sizeof(float));
            TRY_ALLOC(h.bphi[1], h.N * (size_t)h.max_samples * sizeof(float));
        }
    } else {
        TRY_ALLOC(h.b0, h.N * sb);
        TRY_ALLOC(h.dfx, h.N * sizeof(double));
        TRY_ALLOC(h.dfy, h.N * sizeof(double));
        TRY_ALLOC(h.dfz, h.N * sizeof(double));
    }
    h.bwork_bytes = gbg::bwork_total(h);
    TRY_ALLOC(h.bwork, h.bwork_bytes);
    TRY_ALLOC(h.dev_status, sizeof(int));
    TRY_ALLOC(h.barrier, 4 * sizeof(unsigned));
#undef TRY_ALLOC
    if (cudaMemset(h.dev_status, 0, sizeof(int)) != cudaSuccess ||
        cudaMemset(h.barrier, 0, 4 * sizeof(unsigned)) != cudaSuccess) {
        set_error("memset failed");
        return fail(GBG_ERR_CUDA);
    }
    *out = hh;
    return GBG_OK;
}

int gbg_destroy(gbg_handle *hh) {
    if (!hh) return GBG_OK;
    cudaSetDevice(hh->h.device);
    if (hh->h.stream) cudaStreamSynchronize(hh->h.stream);
    free_handle(hh->h);
    delete hh;
    return GBG_OK;
}

int gbg_set_anatomy(gbg_handle *hh, const double *p_w, const double *p_g) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!p_w || !p_g) {
        set_error("null field");
        return GBG_ERR_ARG;
    }
    if (!all_finite(p_w, h.N) || !all_finite(p_g, h.N)) {
        set_error("anatomy has NaN or Inf");
        return GBG_ERR_NONFINITE;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    GBG_CUDA_TRY(cudaMemcpyAsync(h.pw, p_w, h.N * sizeof(double), cudaMemcpyHostToDevice, h.stream));
    GBG_CUDA_TRY(cudaMemcpyAsync(h.pg, p_g, h.N * sizeof(double), cudaMemcpyHostToDevice, h.stream));
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    h.anatomy_set = true;
    h.tables_valid = false;
    h.fast_valid = false;
    h.live_valid = false;
    h.mala_valid = false;
    ++h.state_gen;
    return GBG_OK;
}

int gbg_set_phi(gbg_handle *hh, const double *phi) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!phi) {
        set_error("null field");
        return GBG_ERR_ARG;
    }
    if (!all_finite(phi, h.N)) {
        set_error("phi has NaN or Inf");
        return GBG_ERR_NONFINITE;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    h.cur = 0;
    if (h.prec == GBG_PREC_F64) {
        GBG_CUDA_TRY(cudaMemcpyAsync(h.phi[0], phi, h.N * sizeof(double), cudaMemcpyHostToDevice, h.stream));
    } else {
        std::vector<float> tmp(h.N);
        for (size_t i = 0; i < h.N; ++i) tmp[i] = (float)phi[i];
        GBG_CUDA_TRY(cudaMemcpyAsync(h.phi[0], tmp.data(), h.N * sizeof(float), cudaMemcpyHostToDevice, h.stream));
        GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    }
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    h.phi_set = true;
    return GBG_OK;
}

int gbg_get_phi(gbg_handle *hh, double *phi) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!phi) {
        set_error("null field");
        return GBG_ERR_ARG;
    }
    if (!h.phi_set) {
        set_error("phi not set");
        return GBG_ERR_STATE;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    if (h.prec == GBG_PREC_F64) {
        GBG_CUDA_TRY(cudaMemcpyAsync(phi, h.phi[h.cur], h.N * sizeof(double), cudaMemcpyDeviceToHost, h.stream));
        GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    } else {
        std::vector<float> tmp(h.N);
        GBG_CUDA_TRY(cudaMemcpyAsync(tmp.data(), h.phi[h.cur], h.N * sizeof(float), cudaMemcpyDeviceToHost, h.stream));
        GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
        for (size_t i = 0; i < h.N; ++i) phi[i] = (double)tmp[i];
    }
    return GBG_OK;
}

int gbg_rd_step(gbg_handle *hh, double Dw, double Dg, double rho, double dt, long nsteps) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!h.anatomy_set || !h.phi_set) {
        set_error("set anatomy and phi before stepping");
        return GBG_ERR_STATE;
    }
    if (nsteps < 0 || !std::isfinite(Dw) || !std::isfinite(Dg) || !std::isfinite(rho) ||
        !std::isfinite(dt) || !(Dw > 0) || !(Dg >= 0) || !(dt > 0)) {
        set_error("bad step parameters");
        return GBG_ERR_ARG;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    if (h.prec == GBG_PREC_F32) {
        int rc = gbg::fast_build_tables(h, (double)(float)(Dg / Dw));
        if (rc) return rc;
        return gbg::fast_steps_single(h, Dw, rho, dt, nsteps);
    }
    return gbg::exact_steps(h, Dw, Dg, rho, dt, nsteps);
}

int gbg_population_variant_name(gbg_handle *hh, int index, char *buf, int len) {
    if (int rc = check_handle(hh)) return rc;
    if (gbg::population_variant_name(hh->h.n, index, buf, len) != GBG_OK) {
        set_error("variant index out of range or no buffer");
        return GBG_ERR_ARG;
    }
    return GBG_OK;
}

namespace {

// slopes and the slopes' tissue tensor, allocated on first use (exact modes)
int ensure_mala(Handle &h) {
    if (h.prec == GBG_PREC_F32) {
        set_error("the MALA variant runs in GBG_PREC_F64 or GBG_PREC_F32REF");
        return GBG_ERR_UNSUPPORTED;
    }
    const size_t sb = storage_bytes(h.prec);
    for (int k = 0; k < 2; ++k) {
        if (!h.sr[k]) GBG_CUDA_TRY(cudaMalloc(&h.sr[k], h.N * sb));
        if (!h.sd[k]) GBG_CUDA_TRY(cudaMalloc(&h.sd[k], h.N * sb));
    }
    if (!h.mala_tt) GBG_CUDA_TRY(cudaMalloc((void **)&h.mala_tt, 6 * h.N * sizeof(double)));
    return GBG_OK;
}

}  // namespace

int gbg_set_slopes(gbg_handle *hh, const double *sRho, const double *sD) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if ((sRho && !all_finite(sRho, h.N)) || (sD && !all_finite(sD, h.N))) {
        set_error("slopes have NaN or Inf");
        return GBG_ERR_NONFINITE;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    if (int rc = ensure_mala(h)) return rc;
    const size_t sb = storage_bytes(h.prec);
    const double *src[2] = {sRho, sD};
    void *dst[2] = {h.sr[h.cur], h.sd[h.cur]};
    for (int k = 0; k < 2; ++k) {
        if (!src[k]) {
            GBG_CUDA_TRY(cudaMemsetAsync(dst[k], 0, h.N * sb, h.stream));
        } else if (h.prec == GBG_PREC_F64) {
            GBG_CUDA_TRY(cudaMemcpyAsync(dst[k], src[k], h.N * sizeof(double), cudaMemcpyHostToDevice, h.stream));
            GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
        } else {
            std::vector<float> tmp(h.N);
            for (size_t i = 0; i < h.N; ++i) tmp[i] = (float)src[k][i];
            GBG_CUDA_TRY(cudaMemcpyAsync(dst[k], tmp.data(), h.N * sizeof(float), cudaMemcpyHostToDevice, h.stream));
            GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
        }
    }
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    h.slopes_set = true;
    return GBG_OK;
}

int gbg_get_slopes(gbg_handle *hh, double *sRho, double *sD) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!sRho || !sD) {
        set_error("null field");
        return GBG_ERR_ARG;
    }
    if (!h.slopes_set) {
        set_error("slopes not set");
        return GBG_ERR_STATE;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    double *dst[2] = {sRho, sD};
    void *src[2] = {h.sr[h.cur], h.sd[h.cur]};
    for (int k = 0; k < 2; ++k) {
        if (h.prec == GBG_PREC_F64) {
            GBG_CUDA_TRY(cudaMemcpyAsync(dst[k], src[k], h.N * sizeof(double), cudaMemcpyDeviceToHost, h.stream));
            GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
        } else {
            std::vector<float> tmp(h.N);
            GBG_CUDA_TRY(cudaMemcpyAsync(tmp.data(), src[k], h.N * sizeof(float), cudaMemcpyDeviceToHost, h.stream));
            GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
            for (size_t i = 0; i < h.N; ++i) dst[k][i] = (double)tmp[i];
        }
    }
    return GBG_OK;
}

int gbg_mala_step(gbg_handle *hh, double Dw, double Dg, double rho, double dt, long nsteps) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!h.anatomy_set || !h.phi_set) {
        set_error("set anatomy and phi before stepping");
        return GBG_ERR_STATE;
    }
    if (nsteps < 0 || !std::isfinite(Dw) || !std::isfinite(Dg) || !std::isfinite(rho) ||
        !std::isfinite(dt) || !(Dw > 0) || !(Dg >= 0) || !(dt > 0)) {
        set_error("bad step parameters");
        return GBG_ERR_ARG;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    if (!h.slopes_set)
        if (int rc = gbg_set_slopes(hh, nullptr, nullptr)) return rc;
    if (int rc = ensure_mala(h)) return rc;
    return gbg::mala_steps(h, Dw, Dg, rho, dt, nsteps);
}

int gbg_run_mala(gbg_handle *hh, double Dw_file, double rho, double tend, double L, long *nsteps_out,
                 double *dt_out) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!std::isfinite(Dw_file) || !std::isfinite(rho) || !std::isfinite(tend) || !(L > 0) ||
        !(Dw_file > 0)) {
        set_error("bad run parameters");
        return GBG_ERR_ARG;
    }
    if (h.prec == GBG_PREC_F32) {
        set_error("the MALA variant runs in GBG_PREC_F64 or GBG_PREC_F32REF");
        return GBG_ERR_UNSUPPORTED;
    }
    double dt, Dw, Dg, r = rho;
    gbg::reference_dt(h.n, Dw_file, L, h.prec == GBG_PREC_F32REF, &dt, &Dw, &Dg, &r);
    const long ns = gbg::reference_num_steps(dt, tend);
    if (nsteps_out) *nsteps_out = ns;
    if (dt_out) *dt_out = dt;
    int rc = gbg_mala_step(hh, Dw, Dg, r, dt, ns);
    if (rc) return rc;
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    return GBG_OK;
}

int gbg_run(gbg_handle *hh, double Dw_file, double rho, double tend, double L, long *nsteps_out,
            double *dt_out) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!std::isfinite(Dw_file) || !std::isfinite(rho) || !std::isfinite(tend) || !(L > 0) ||
        !(Dw_file > 0)) {
        set_error("bad run parameters");
        return GBG_ERR_ARG;
    }
    double dt, Dw, Dg, r = rho;
    // the fast path keeps the double-precision timeline of the FP64 reference
    gbg::reference_dt(h.n, Dw_file, L, h.prec == GBG_PREC_F32REF, &dt, &Dw, &Dg, &r);
    const long ns = gbg::reference_num_steps(dt, tend);
    if (nsteps_out) *nsteps_out = ns;
    if (dt_out) *dt_out = dt;
    int rc = gbg_rd_step(hh, Dw, Dg, r, dt, ns);
    if (rc) return rc;
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    return GBG_OK;
}

int gbg_set_observations(gbg_handle *hh, const double *pet, const double *t1, const double *t2,
                         const double *points, long npoints, const gbg_lik_params *p) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!pet || !t1 || !t2 || !p || (p->selective && (npoints < 0 || (npoints > 0 && !points)))) {
        set_error("null observation argument");
        return GBG_ERR_ARG;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    return gbg::lik_set_observations(h, pet, t1, t2, points, npoints, *p);
}

int gbg_loglik(gbg_handle *hh, gbg_lik_result *out) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!out) {
        set_error("null output");
        return GBG_ERR_ARG;
    }
    if (!h.phi_set) {
        set_error("phi not set");
        return GBG_ERR_STATE;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    if (int rc = ensure_lik_out(h, 1)) return rc;
    int rc;
    if (h.prec == GBG_PREC_F64)
        rc = gbg::lik_evaluate(h, nullptr, (const double *)h.phi[h.cur], 1, (gbg_lik_result *)h.lik_out);
    else
        rc = gbg::lik_evaluate(h, (const float *)h.phi[h.cur], nullptr, 1, (gbg_lik_result *)h.lik_out);
    if (rc) return rc;
    GBG_CUDA_TRY(cudaMemcpyAsync(out, h.lik_out, sizeof(gbg_lik_result), cudaMemcpyDeviceToHost, h.stream));
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    return GBG_OK;
}

static int validate_batch(Handle &h, int S, const gbg_batch_opts *o) {
    if (!o || S <= 0 || S > h.max_samples || !(o->L > 0) || !(o->ic_sigma > 0) ||
        !std::isfinite(o->ic_peak) || !std::isfinite(o->dt0) || o->dt0 < -1.0) {
        set_error("bad batch arguments");
        return GBG_ERR_ARG;
    }
    if (!h.anatomy_set) {
        set_error("anatomy not set");
        return GBG_ERR_STATE;
    }
    if (o->with_loglik && !h.obs.valid) {
        set_error("observations not set");
        return GBG_ERR_STATE;
    }
    return GBG_OK;
}

int gbg_batch_solve_device(gbg_handle *hh, const gbg_sample *samples_device, int S,
                           const gbg_batch_opts *o, gbg_lik_result *loglik_device) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (int rc = validate_batch(h, S, o)) return rc;
    if (!samples_device) {
        set_error("null samples");
        return GBG_ERR_ARG;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    return gbg::batch_solve_device(h, samples_device, S, *o, loglik_device, nullptr);
}

int gbg_set_batch_graphs(gbg_handle *hh, int enabled) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    h.batch_graphs = enabled != 0;
    if (!h.batch_graphs) {
        GBG_CUDA_TRY(cudaSetDevice(h.device));
        GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
        gbg::batch_graphs_clear(h);
    }
    return GBG_OK;
}

int gbg_batch_solve(gbg_handle *hh, const gbg_sample *samples, int S, const gbg_batch_opts *o,
                    gbg_lik_result *loglik, long *nsteps_out, float *phi_out) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (int rc = validate_batch(h, S, o)) return rc;
    if (!samples) {
        set_error("null samples");
        return GBG_ERR_ARG;
    }
    for (int s = 0; s < S; ++s) {
        const gbg_sample &q = samples[s];
        if (!std::isfinite(q.Dw) || !(q.Dw > 0) || !std::isfinite(q.rho) || !std::isfinite(q.x0) ||
            !std::isfinite(q.y0) || !std::isfinite(q.z0) || !std::isfinite(q.tend)) {
            set_error("non-finite or non-positive sample parameter");
            return GBG_ERR_NONFINITE;
        }
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    gbg_sample *d_samples = gbg::batch_samples(h);
    GBG_CUDA_TRY(cudaMemcpyAsync(d_samples, samples, sizeof(gbg_sample) * S, cudaMemcpyHostToDevice, h.stream));
    gbg_lik_result *d_lik = nullptr;
    if (o->with_loglik) {
        // sized for max_samples at once: captured graphs name this buffer
        if (int rc = ensure_lik_out(h, std::max(S, h.max_samples))) return rc;
        d_lik = (gbg_lik_result *)h.lik_out;
    }
    // one graph launch per call (captured on the first call with this S and
    // these options) unless graphs are switched off for the handle
    int rc = (h.batch_graphs && h.prec == GBG_PREC_F32)
                 ? gbg::batch_graph_run(h, d_samples, S, *o, d_lik)
                 : gbg::batch_solve_device(h, d_samples, S, *o, d_lik, nullptr);
    if (rc) return rc;
    std::vector<gbg::SampleRec> recs(S);
    GBG_CUDA_TRY(cudaMemcpyAsync(recs.data(), gbg::batch_unsorted(h), sizeof(gbg::SampleRec) * S,
                                 cudaMemcpyDeviceToHost, h.stream));
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    rc = gbg::check_device_status(h);
    if (rc) return rc;
    std::vector<long> steps(S);
    for (int s = 0; s < S; ++s) steps[s] = recs[s].nsteps;
    if (nsteps_out)
        for (int s = 0; s < S; ++s) nsteps_out[s] = steps[s];
    if (loglik && d_lik)
        GBG_CUDA_TRY(cudaMemcpyAsync(loglik, d_lik, sizeof(gbg_lik_result) * S, cudaMemcpyDeviceToHost, h.stream));
    if (phi_out) {
        for (int s = 0; s < S; ++s) {
            const float *src = h.bphi[steps[s] & 1] + (size_t)s * h.N;
            GBG_CUDA_TRY(cudaMemcpyAsync(phi_out + (size_t)s * h.N, src, h.N * sizeof(float),
                                         cudaMemcpyDeviceToHost, h.stream));
        }
    }
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    return GBG_OK;
}

int gbg_batch_statistics(gbg_handle *hh, const gbg_sample *samples, int S, const gbg_batch_opts *o,
                         int reference_rules, double *mean, double *var) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (int rc = validate_batch(h, S, o)) return rc;
    if (!samples || !mean || !var) {
        set_error("null samples or outputs");
        return GBG_ERR_ARG;
    }
    for (int s = 0; s < S; ++s) {
        const gbg_sample &q = samples[s];
        if (!std::isfinite(q.Dw) || !(q.Dw > 0) || !std::isfinite(q.rho) || !std::isfinite(q.x0) ||
            !std::isfinite(q.y0) || !std::isfinite(q.z0) || !std::isfinite(q.tend)) {
            set_error("non-finite or non-positive sample parameter");
            return GBG_ERR_NONFINITE;
        }
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    gbg_sample *d_samples = gbg::batch_samples(h);
    GBG_CUDA_TRY(cudaMemcpyAsync(d_samples, samples, sizeof(gbg_sample) * S, cudaMemcpyHostToDevice, h.stream));
    float *d = nullptr;
    GBG_CUDA_TRY(cudaMalloc((void **)&d, 2 * h.N * sizeof(float)));
    gbg_batch_opts oo = *o;
    oo.with_loglik = 0;
    int rc = gbg::batch_statistics(h, d_samples, S, oo, reference_rules, d, d + h.N);
    if (!rc) rc = gbg::check_device_status(h);
    std::vector<float> tmp(2 * h.N);
    if (!rc && cudaMemcpyAsync(tmp.data(), d, 2 * h.N * sizeof(float), cudaMemcpyDeviceToHost, h.stream) !=
                   cudaSuccess)
        rc = GBG_ERR_CUDA;
    if (!rc && cudaStreamSynchronize(h.stream) != cudaSuccess) rc = GBG_ERR_CUDA;
    cudaFree(d);
    if (rc) {
        if (rc == GBG_ERR_CUDA) set_error("gbg_batch_statistics: CUDA error");
        return rc;
    }
    for (size_t c = 0; c < h.N; ++c) {
        mean[c] = tmp[c];
        var[c] = tmp[h.N + c];
    }
    return GBG_OK;
}

int gbg_adjoint_grad(gbg_handle *hh, const gbg_sample *samples, int S, const gbg_adjoint_opts *o,
                     double *loglik, double *grad) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (h.is_amr) {
        set_error("the adjoint runs on uniform-grid handles");
        return GBG_ERR_STATE;
    }
    if (!samples || S < 1 || !o || !(o->dt0 != 0) || !std::isfinite(o->dt0) || o->dt0 < -1.0 || !(o->L > 0) ||
        !(o->ic_sigma > 0) ||
        o->checkpoint_every < 0 || (o->state_precision != GBG_PREC_F32 && o->state_precision != GBG_PREC_F64)) {
        set_error("bad adjoint arguments");
        return GBG_ERR_ARG;
    }
    for (int s = 0; s < S; ++s)
        if (!std::isfinite(samples[s].Dw) || !std::isfinite(samples[s].rho) || !std::isfinite(samples[s].tend) ||
            !(samples[s].Dw > 0) || !(samples[s].tend > 0) ||
            samples[s].tend / (o->dt0 > 0 ? o->dt0
                                          : -o->dt0 * 0.99 /
                                                (6.0 * h.n * h.n * samples[s].Dw / (o->L * o->L) +
                                                 0.5 * std::fabs(samples[s].rho))) >
                1e6) {
            set_error("non-finite or out-of-range sample parameter");
            return GBG_ERR_NONFINITE;
        }
    if (!h.anatomy_set || !h.obs.valid) {
        set_error("set anatomy and observations first");
        return GBG_ERR_STATE;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    int rc = gbg::adjoint_grad(h, samples, S, *o, loglik, grad);
    // the forward sweep's population kernel reports a barrier timeout here
    if (!rc) rc = gbg::check_device_status(h);
    return rc;
}

int gbg_amr_create(const gbg_amr_config *cfg, gbg_handle **out) {
    if (!cfg || !out) {
        set_error("null argument");
        return GBG_ERR_ARG;
    }
    *out = nullptr;
    if (cfg->max_blocks < 1 || (cfg->precision != GBG_PREC_F64 && cfg->precision != GBG_PREC_F32REF &&
                                cfg->precision != GBG_PREC_F32)) {
        set_error("bad AMR configuration (max_blocks >= 1; GBG_PREC_F64, GBG_PREC_F32REF or GBG_PREC_F32)");
        return GBG_ERR_ARG;
    }
    int ndev = 0;
    GBG_CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (cfg->device < 0 || cfg->device >= ndev) {
        set_error("device ordinal out of range");
        return GBG_ERR_ARG;
    }
    GBG_CUDA_TRY(cudaSetDevice(cfg->device));
    gbg_handle *hh = new gbg_handle();
    Handle &h = hh->h;
    h.is_amr = true;
    h.prec = cfg->precision;
    h.device = cfg->device;
    h.amr.max_blocks = cfg->max_blocks;
    if (cudaDeviceGetAttribute(&h.num_sms, cudaDevAttrMultiProcessorCount, h.device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h.stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete hh;
        set_error("stream creation failed");
        return GBG_ERR_CUDA;
    }
    if (int rc = gbg::amr_alloc(h)) {
        free_handle(h);
        delete hh;
        return rc;
    }
    *out = hh;
    return GBG_OK;
}

static int check_amr(gbg_handle *hh) {
    if (int rc = check_handle(hh)) return rc;
    if (!hh->h.is_amr) {
        set_error("not a handle made by gbg_amr_create");
        return GBG_ERR_STATE;
    }
    return GBG_OK;
}

int gbg_amr_set_grid(gbg_handle *hh, int nb, const gbg_block *blocks, const double *p_w, const double *p_g,
                     const double *phi) {
    if (int rc = check_amr(hh)) return rc;
    Handle &h = hh->h;
    if (nb < 1 || nb > h.amr.max_blocks || !blocks || !p_w || !p_g || !phi) {
        set_error("bad grid arguments");
        return GBG_ERR_ARG;
    }
    for (int i = 0; i < nb; ++i) {
        const gbg_block &b = blocks[i];
        const int side = b.level >= 0 && b.level < 16 ? 1 << b.level : -1;
        if (side < 0 || b.ix < 0 || b.iy < 0 || b.iz < 0 || b.ix >= side || b.iy >= side || b.iz >= side) {
            set_error("block position outside its level");
            return GBG_ERR_ARG;
        }
    }
    const size_t n = (size_t)nb * 4096;
    if (!all_finite(p_w, n) || !all_finite(p_g, n) || !all_finite(phi, n)) {
        set_error("grid fields have NaN or Inf");
        return GBG_ERR_NONFINITE;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    return gbg::amr_set_grid(h, nb, blocks, p_w, p_g, phi);
}

int gbg_amr_set_ghosts(gbg_handle *hh, const long *start, const int *src_block, const int *src_cell,
                       const double *w, long nentries) {
    if (int rc = check_amr(hh)) return rc;
    Handle &h = hh->h;
    if (h.amr.nb < 1) {
        set_error("set the grid before its ghost tables");
        return GBG_ERR_STATE;
    }
    if (!start || nentries < 0 || (nentries > 0 && (!src_block || !src_cell || !w))) {
        set_error("bad ghost-table arguments");
        return GBG_ERR_ARG;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    return gbg::amr_set_ghosts(h, start, src_block, src_cell, w, nentries);
}

int gbg_amr_step(gbg_handle *hh, double Dw, double Dg, double rho, double dt, long nsteps) {
    if (int rc = check_amr(hh)) return rc;
    if (nsteps < 0 || !std::isfinite(Dw) || !std::isfinite(Dg) || !std::isfinite(rho) || !std::isfinite(dt)) {
        set_error("bad step parameters");
        return GBG_ERR_ARG;
    }
    GBG_CUDA_TRY(cudaSetDevice(hh->h.device));
    return gbg::amr_steps(hh->h, Dw, Dg, rho, dt, nsteps);
}

int gbg_amr_fast_variant(gbg_handle *hh, int variant) {
    if (int rc = check_amr(hh)) return rc;
    if (variant < 0 || variant > 1) {
        set_error("fast variant: 0 (fused) or 1 (separate ghost pass)");
        return GBG_ERR_ARG;
    }
    if (hh->h.amr.fast_variant != variant) hh->h.amr.tables_valid = false;  // the layouts differ
    hh->h.amr.fast_variant = variant;
    return GBG_OK;
}

int gbg_amr_get_phi(gbg_handle *hh, double *phi) {
    if (int rc = check_amr(hh)) return rc;
    if (!phi || hh->h.amr.nb < 1) {
        set_error("bad arguments or no grid");
        return GBG_ERR_ARG;
    }
    GBG_CUDA_TRY(cudaSetDevice(hh->h.device));
    return gbg::amr_get_phi(hh->h, phi);
}

int gbg_amr_fwt_detail(gbg_handle *hh, double *detail) {
    if (int rc = check_amr(hh)) return rc;
    if (!detail) {
        set_error("null output");
        return GBG_ERR_ARG;
    }
    GBG_CUDA_TRY(cudaSetDevice(hh->h.device));
    return gbg::amr_fwt_detail(hh->h, detail);
}

int gbg_amr_remap(gbg_handle *hh, int nbn, const gbg_block *blocks, const int *kind, const int *src) {
    if (int rc = check_amr(hh)) return rc;
    Handle &h = hh->h;
    if (nbn < 1 || nbn > h.amr.max_blocks || !blocks || !kind || !src) {
        set_error("bad remap arguments");
        return GBG_ERR_ARG;
    }
    for (int i = 0; i < nbn; ++i) {
        const int *s = src + 8 * (size_t)i;
        const int nsrc = kind[i] == GBG_REMAP_COLLAPSE ? 8 : 1;
        if (kind[i] < GBG_REMAP_COPY || kind[i] > GBG_REMAP_COLLAPSE ||
            (kind[i] == GBG_REMAP_SPLIT && (s[1] < 0 || s[1] > 7))) {
            set_error("bad remap kind or child index");
            return GBG_ERR_ARG;
        }
        for (int k = 0; k < nsrc; ++k)
            if (s[k] < 0 || s[k] >= h.amr.nb) {
                set_error("remap source outside the current grid");
                return GBG_ERR_ARG;
            }
        const int side = blocks[i].level >= 0 && blocks[i].level < 16 ? 1 << blocks[i].level : -1;
        if (side < 0 || blocks[i].ix < 0 || blocks[i].iy < 0 || blocks[i].iz < 0 || blocks[i].ix >= side ||
            blocks[i].iy >= side || blocks[i].iz >= side) {
            set_error("block position outside its level");
            return GBG_ERR_ARG;
        }
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    return gbg::amr_remap(h, nbn, blocks, kind, src);
}

int gbg_amr_build_ghosts(gbg_handle *hh) {
    if (int rc = check_amr(hh)) return rc;
    if (hh->h.amr.nb < 1) {
        set_error("set the grid first");
        return GBG_ERR_STATE;
    }
    GBG_CUDA_TRY(cudaSetDevice(hh->h.device));
    return gbg::amr_build_ghosts(hh->h);
}

int gbg_amr_auto_refine(gbg_handle *hh, double tol, int max_level, int *nrefined) {
    if (int rc = check_amr(hh)) return rc;
    if (!nrefined || !(tol >= 0) || hh->h.amr.nb < 1) {
        set_error("bad refinement arguments (set the grid first)");
        return GBG_ERR_ARG;
    }
    GBG_CUDA_TRY(cudaSetDevice(hh->h.device));
    if (!hh->h.amr.ghosts_valid)
        if (int rc = gbg::amr_build_ghosts(hh->h)) return rc;
    return gbg::amr_auto_refine(hh->h, tol, max_level, nrefined);
}

int gbg_amr_auto_compress(gbg_handle *hh, double tol, int *ncollapsed) {
    if (int rc = check_amr(hh)) return rc;
    if (!ncollapsed || !(tol >= 0) || hh->h.amr.nb < 1) {
        set_error("bad compression arguments (set the grid first)");
        return GBG_ERR_ARG;
    }
    GBG_CUDA_TRY(cudaSetDevice(hh->h.device));
    if (!hh->h.amr.ghosts_valid)
        if (int rc = gbg::amr_build_ghosts(hh->h)) return rc;
    return gbg::amr_auto_compress(hh->h, tol, ncollapsed);
}

int gbg_amr_get_blocks(gbg_handle *hh, gbg_block *blocks, int capacity, int *nblocks) {
    if (int rc = check_amr(hh)) return rc;
    if (!nblocks) {
        set_error("null output");
        return GBG_ERR_ARG;
    }
    const std::vector<gbg_block> &b = hh->h.amr.hblocks;
    *nblocks = (int)b.size();
    if (!blocks) return GBG_OK;
    if (capacity < (int)b.size()) {
        set_error("capacity below the block count (see *nblocks)");
        return GBG_ERR_ARG;
    }
    std::copy(b.begin(), b.end(), blocks);
    return GBG_OK;
}

int gbg_amr_run(gbg_handle *hh, const gbg_amr_run_opts *o, long *steps, int *regrids) {
    if (int rc = check_amr(hh)) return rc;
    if (!o || !steps || !regrids || hh->h.amr.nb < 1 || !std::isfinite(o->Dw_file) || !(o->Dw_file > 0) ||
        !std::isfinite(o->rho) || !std::isfinite(o->tend) || !(o->L > 0) || o->bpd < 1 ||
        (o->adaptive && (!(o->dumpfreq > 0) || !(o->refine_tol >= 0) || !(o->compress_tol >= 0)))) {
        set_error("bad adaptive-run arguments (set the grid first)");
        return GBG_ERR_ARG;
    }
    double dt, Dw, Dg, rho = o->rho;
    gbg::reference_dt(16 * o->bpd, o->Dw_file, o->L, false, &dt, &Dw, &Dg, &rho);
    if (o->tend / dt > 1e8) {
        set_error("too many steps (tend / dt > 1e8)");
        return GBG_ERR_ARG;
    }
    GBG_CUDA_TRY(cudaSetDevice(hh->h.device));
    return gbg::amr_run(hh->h, *o, steps, regrids);
}

int gbg_amr_last_run_stats(gbg_handle *hh, gbg_amr_run_stats *stats) {
    if (int rc = check_amr(hh)) return rc;
    if (!stats) {
        set_error("null output");
        return GBG_ERR_ARG;
    }
    *stats = hh->h.amr.last_run;
    return GBG_OK;
}

int gbg_amr_dump_uniform(gbg_handle *hh, int gpd, int reference_rules, double *out) {
    if (int rc = check_amr(hh)) return rc;
    if (gpd < 1 || gpd > 2048 || (gpd & (gpd - 1)) || !out || hh->h.amr.nb < 1) {
        set_error("bad dump arguments (gpd a power of two)");
        return GBG_ERR_ARG;
    }
    GBG_CUDA_TRY(cudaSetDevice(hh->h.device));
    return gbg::amr_dump_uniform(hh->h, gpd, reference_rules, out);
}

}  // extern "C"

extern "C" {

int gbg_affine_set(gbg_handle *hh, int P, const float *phi0, const float *J) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!phi0 || !J) {
        set_error("null field");
        return GBG_ERR_ARG;
    }
    if (h.is_amr || h.prec != GBG_PREC_F32 || !h.anatomy_set) {
        set_error("affine model needs a GBG_PREC_F32 handle with its anatomy set");
        return GBG_ERR_STATE;
    }
    for (size_t i = 0; i < h.N; ++i)
        if (!std::isfinite(phi0[i])) {
            set_error("phi0 has NaN or Inf");
            return GBG_ERR_NONFINITE;
        }
    if (P >= 1 && P <= 16)
        for (size_t i = 0; i < (size_t)P * h.N; ++i)
            if (!std::isfinite(J[i])) {
                set_error("J has NaN or Inf");
                return GBG_ERR_NONFINITE;
            }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    return gbg::affine_set(h, P, phi0, J);
}

int gbg_affine_loglik(gbg_handle *hh, int B, const double *delta, gbg_lik_result *out) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!delta || !out || B < 1) {
        set_error("bad affine arguments");
        return GBG_ERR_ARG;
    }
    if (!h.obs.valid) {
        set_error("observations not set");
        return GBG_ERR_STATE;
    }
    for (size_t i = 0; i < (size_t)B * (h.aff_P > 0 ? h.aff_P : 0); ++i)
        if (!std::isfinite(delta[i])) {
            set_error("non-finite delta");
            return GBG_ERR_NONFINITE;
        }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    if (int rc = ensure_lik_out(h, B)) return rc;
    if (int rc = gbg::affine_loglik(h, B, delta, (gbg_lik_result *)h.lik_out)) return rc;
    GBG_CUDA_TRY(cudaMemcpyAsync(out, h.lik_out, B * sizeof(gbg_lik_result), cudaMemcpyDeviceToHost, h.stream));
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    return GBG_OK;
}

int gbg_observation_counts(gbg_handle *hh, long *n_pet, long *n_ti) {
    if (int rc = check_handle(hh)) return rc;
    if (!n_pet || !n_ti) {
        set_error("null output");
        return GBG_ERR_ARG;
    }
    if (!hh->h.obs.valid) {
        set_error("observations not set");
        return GBG_ERR_STATE;
    }
    *n_pet = hh->h.obs.n_pet;
    *n_ti = hh->h.obs.n_ti;
    return GBG_OK;
}

int gbg_affine_set_prior_mask(gbg_handle *hh, const unsigned char *mask) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!mask) {
        set_error("null mask");
        return GBG_ERR_ARG;
    }
    if (h.is_amr) {
        set_error("affine chain needs a uniform-grid handle");
        return GBG_ERR_STATE;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    return gbg::affine_set_prior_mask(h, mask);
}

int gbg_affine_chain(gbg_handle *hh, const gbg_affine_chain_opts *o, int B, int steps, unsigned long long seed,
                     double *v, double *lp_start, double *lp_end, int *counts) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!o || !v || !lp_start || !lp_end || B < 1 || B > 65535 || steps < 0) {
        set_error("bad affine chain arguments");
        return GBG_ERR_ARG;
    }
    if (o->axis < -1 || o->axis > 5 || o->quad_axis < -1 || o->quad_axis > 5 || !(o->axis_prob >= 0) ||
        !(o->axis_prob <= 1) || !std::isfinite(o->step) || o->log_mask < 0 || o->log_mask > 63 ||
        !(o->ind_prob >= 0) || !(o->ind_prob + (o->axis >= 0 ? o->axis_prob : 0.0) <= 1)) {
        set_error("affine chain options out of range");
        return GBG_ERR_ARG;
    }
    for (int i = 0; i < 36; ++i)
        if (!std::isfinite(o->chol[i]) || !std::isfinite(o->Ai[i]) || !std::isfinite(o->ind_chol[i]) ||
            !std::isfinite(o->ind_inv[i])) {
            set_error("non-finite affine chain matrix");
            return GBG_ERR_NONFINITE;
        }
    for (int i = 0; i < 6; ++i) {
        const bool lg = (o->log_mask >> i) & 1;
        if (!std::isfinite(o->u_ref[i]) || !std::isfinite(o->lo[i]) || !std::isfinite(o->hi[i]) ||
            !std::isfinite(o->ind_mean[i]) ||
            !(o->hi[i] > o->lo[i]) || (lg && !(o->lo[i] > 0))) {
            set_error("bad affine chain prior box or centre");
            return GBG_ERR_ARG;
        }
        // the redrawn coordinate may move log coordinates only
        if (o->axis >= 0 && !lg && o->Ai[i * 6 + o->axis] != 0) {
            set_error("the redrawn coordinate moves a non-log coordinate");
            return GBG_ERR_ARG;
        }
    }
    for (size_t i = 0; i < (size_t)B * 6; ++i)
        if (!std::isfinite(v[i])) {
            set_error("non-finite chain state");
            return GBG_ERR_NONFINITE;
        }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    return gbg::affine_chain(h, *o, B, steps, seed, v, lp_start, lp_end, counts);
}

}  // extern "C"

struct gbg_surrogate {
    gbg::Surrogate *s;
    gbg_handle *owner;
};

extern "C" {

int gbg_surrogate_create(gbg_handle *hh, const gbg_surrogate_config *cfg, gbg_surrogate **out) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!cfg || !out) {
        set_error("null argument");
        return GBG_ERR_ARG;
    }
    *out = nullptr;
    if (h.is_amr || h.prec != GBG_PREC_F32 || h.max_samples < 1 || !h.anatomy_set) {
        set_error("surrogate needs a GBG_PREC_F32 handle with max_samples >= 1 and its anatomy set");
        return GBG_ERR_STATE;
    }
    if (!(cfg->L > 0) || !(cfg->dw_hi > cfg->dw_lo) || !(cfg->rho_hi > cfg->rho_lo) || !(cfg->t_hi > cfg->t_lo)) {
        set_error("bad surrogate configuration");
        return GBG_ERR_ARG;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    gbg::Surrogate *s = nullptr;
    if (int rc = gbg::surrogate_create(h, *cfg, &s)) return rc;
    *out = new gbg_surrogate{s, hh};
    return GBG_OK;
}

int gbg_surrogate_destroy(gbg_surrogate *s) {
    if (!s) return GBG_OK;
    gbg::surrogate_destroy(s->s);
    delete s;
    return GBG_OK;
}

static int check_sur(gbg_surrogate *s) {
    if (!s || !s->s) {
        set_error("null surrogate");
        return GBG_ERR_ARG;
    }
    cudaSetDevice(s->owner->h.device);
    return GBG_OK;
}

int gbg_surrogate_nparams(gbg_surrogate *s, long *count) {
    if (int rc = check_sur(s)) return rc;
    if (!count) {
        set_error("null output");
        return GBG_ERR_ARG;
    }
    *count = gbg::surrogate_nparams(*s->s);
    return GBG_OK;
}

int gbg_surrogate_get_params(gbg_surrogate *s, float *p) {
    if (int rc = check_sur(s)) return rc;
    if (!p) {
        set_error("null output");
        return GBG_ERR_ARG;
    }
    return gbg::surrogate_get_params(*s->s, p);
}

int gbg_surrogate_set_params(gbg_surrogate *s, const float *p) {
    if (int rc = check_sur(s)) return rc;
    if (!p) {
        set_error("null input");
        return GBG_ERR_ARG;
    }
    return gbg::surrogate_set_params(*s->s, p);
}

static int check_samples(const gbg_sample *smp, int n) {
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(smp[i].Dw) || !std::isfinite(smp[i].rho) || !std::isfinite(smp[i].x0) ||
            !std::isfinite(smp[i].y0) || !std::isfinite(smp[i].z0) || !std::isfinite(smp[i].tend)) {
            set_error("non-finite sample parameter");
            return GBG_ERR_NONFINITE;
        }
    return GBG_OK;
}

int gbg_surrogate_train(gbg_surrogate *s, const gbg_sample *samples, int S, int epochs, int batch, double lr,
                        unsigned long long seed, double *loss) {
    if (int rc = check_sur(s)) return rc;
    if (!samples || S < 1 || epochs < 0 || !(lr > 0)) {
        set_error("bad training arguments");
        return GBG_ERR_ARG;
    }
    if (int rc = check_samples(samples, S)) return rc;
    return gbg::surrogate_train(*s->s, samples, S, epochs, batch, lr, seed, loss);
}

int gbg_surrogate_loss_grad(gbg_surrogate *s, const gbg_sample *samples, int B, const float *targets, double *loss,
                            float *grad) {
    if (int rc = check_sur(s)) return rc;
    if (!samples || !targets || B < 1 || B > gbg::surrogate_batch_max(*s->s)) {
        set_error("bad loss_grad arguments (1 <= B <= batch_max)");
        return GBG_ERR_ARG;
    }
    if (int rc = check_samples(samples, B)) return rc;
    return gbg::surrogate_loss_grad(*s->s, samples, B, targets, loss, grad);
}

int gbg_surrogate_features(gbg_surrogate *s, const gbg_sample *samples, int B, float *out) {
    if (int rc = check_sur(s)) return rc;
    if (!samples || !out || B < 1 || B > gbg::surrogate_batch_max(*s->s)) {
        set_error("bad features arguments (1 <= B <= batch_max)");
        return GBG_ERR_ARG;
    }
    return gbg::surrogate_features(*s->s, samples, B, out);
}

int gbg_surrogate_loglik(gbg_surrogate *s, const gbg_sample *samples, int B, gbg_lik_result *out, float *phi) {
    if (int rc = check_sur(s)) return rc;
    Handle &h = s->owner->h;
    if (!samples || !out || B < 1 || B > gbg::surrogate_batch_max(*s->s)) {
        set_error("bad loglik arguments (1 <= B <= batch_max)");
        return GBG_ERR_ARG;
    }
    if (!h.obs.valid) {
        set_error("observations not set");
        return GBG_ERR_STATE;
    }
    if (int rc = check_samples(samples, B)) return rc;
    if (int rc = ensure_lik_out(h, B)) return rc;
    gbg_sample *d = gbg::batch_samples(h);
    if (B > (h.max_samples > 1 ? h.max_samples : 1)) {
        set_error("B exceeds the handle's sample capacity");
        return GBG_ERR_ARG;
    }
    GBG_CUDA_TRY(cudaMemcpyAsync(d, samples, B * sizeof(gbg_sample), cudaMemcpyHostToDevice, h.stream));
    if (int rc = gbg::surrogate_predict(*s->s, d, B, (gbg_lik_result *)h.lik_out)) return rc;
    GBG_CUDA_TRY(cudaMemcpyAsync(out, h.lik_out, B * sizeof(gbg_lik_result), cudaMemcpyDeviceToHost, h.stream));
    if (phi)
        GBG_CUDA_TRY(cudaMemcpyAsync(phi, gbg::surrogate_prediction(*s->s), (size_t)B * h.N * sizeof(float), cudaMemcpyDeviceToHost,
                                     h.stream));
    GBG_CUDA_TRY(cudaStreamSynchronize(h.stream));
    return gbg::check_device_status(h);
}

int gbg_surrogate_set_engine(gbg_surrogate *s, int engine) {
    if (int rc = check_sur(s)) return rc;
    return gbg::surrogate_set_engine(*s->s, engine);
}

int gbg_launch_count(gbg_handle *hh, long long *count) {
    if (int rc = check_handle(hh)) return rc;
    if (!count) {
        set_error("null output");
        return GBG_ERR_ARG;
    }
    *count = hh->h.launches;
    return GBG_OK;
}

int gbg_stream(gbg_handle *hh, void **stream) {
    if (int rc = check_handle(hh)) return rc;
    if (!stream) {
        set_error("null output");
        return GBG_ERR_ARG;
    }
    *stream = (void *)hh->h.stream;
    return GBG_OK;
}

int gbg_last_population_ms(gbg_handle *hh, float *ms) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!ms) {
        set_error("null output");
        return GBG_ERR_ARG;
    }
    if (!h.ev_pop_recorded) {
        set_error("no population kernel launched yet");
        return GBG_ERR_STATE;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    GBG_CUDA_TRY(cudaEventSynchronize(h.ev_pop[1]));
    GBG_CUDA_TRY(cudaEventElapsedTime(ms, h.ev_pop[0], h.ev_pop[1]));
    return GBG_OK;
}

int gbg_last_population_cells(gbg_handle *hh, long long *cell_steps) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!cell_steps) {
        set_error("null output");
        return GBG_ERR_ARG;
    }
    if (!h.ev_pop_recorded) {
        set_error("no population kernel launched yet");
        return GBG_ERR_STATE;
    }
    if (!h.pop_tile_cells) {
        set_error("the latest population kernel does not count the tiles it computes");
        return GBG_ERR_UNSUPPORTED;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    GBG_CUDA_TRY(cudaEventSynchronize(h.ev_pop[1]));
    unsigned long long tiles = 0;
    GBG_CUDA_TRY(cudaMemcpy(&tiles, h.barrier + 2, sizeof(tiles), cudaMemcpyDeviceToHost));
    *cell_steps = (long long)tiles * h.pop_tile_cells;
    return GBG_OK;
}

int gbg_population_variants(gbg_handle *hh, int *count) {
    if (int rc = check_handle(hh)) return rc;
    if (!count) {
        set_error("null output");
        return GBG_ERR_ARG;
    }
    *count = gbg::population_variant_count(hh->h.n);
    return GBG_OK;
}

int gbg_set_population_variant(gbg_handle *hh, int index) {
    if (int rc = check_handle(hh)) return rc;
    if (index < 0 || index >= gbg::population_variant_count(hh->h.n)) {
        set_error("variant index out of range");
        return GBG_ERR_ARG;
    }
    hh->h.pop_variant = index;
    return GBG_OK;
}

int gbg_population_variant_shape(gbg_handle *hh, int index, int *rows, int *samples_per_cta,
                                 int *threads) {
    if (int rc = check_handle(hh)) return rc;
    if (!rows || !samples_per_cta || !threads) {
        set_error("null output");
        return GBG_ERR_ARG;
    }
    if (gbg::population_variant_shape(hh->h.n, index, rows, samples_per_cta, threads) != GBG_OK) {
        set_error("variant index out of range");
        return GBG_ERR_ARG;
    }
    return GBG_OK;
}

namespace {

// The tuning cache is a flat JSON object {"key": index, ...}.
std::map<std::string, int> read_tune_cache(const char *path) {
    std::map<std::string, int> m;
    std::ifstream f(path);
    if (!f) return m;
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string t = ss.str();
    size_t i = 0;
    while ((i = t.find('"', i)) != std::string::npos) {
        const size_t j = t.find('"', i + 1);
        if (j == std::string::npos) break;
        const std::string key = t.substr(i + 1, j - i - 1);
        const size_t c = t.find(':', j);
        if (c == std::string::npos) break;
        m[key] = std::atoi(t.c_str() + c + 1);
        i = t.find_first_of(",}", c);
        if (i == std::string::npos) break;
    }
    return m;
}

void write_tune_cache(const char *path, const std::map<std::string, int> &m) {
    FILE *f = std::fopen(path, "w");
    if (!f) return;
    std::fprintf(f, "{");
    bool first = true;
    for (const auto &kv : m) {
        std::fprintf(f, "%s\n \"%s\": %d", first ? "" : ",", kv.first.c_str(), kv.second);
        first = false;
    }
    std::fprintf(f, "\n}\n");
    std::fclose(f);
}

}  // namespace

int gbg_autotune(gbg_handle *hh, int probe_samples, const char *cache_path, int *chosen) {
    if (int rc = check_handle(hh)) return rc;
    Handle &h = hh->h;
    if (!chosen || probe_samples < 1 || probe_samples > h.max_samples) {
        set_error("bad autotune arguments (1 <= probe_samples <= max_samples)");
        return GBG_ERR_ARG;
    }
    if (h.prec != GBG_PREC_F32) {
        set_error("autotune applies to GBG_PREC_F32");
        return GBG_ERR_UNSUPPORTED;
    }
    if (!h.anatomy_set) {
        set_error("anatomy not set");
        return GBG_ERR_STATE;
    }
    GBG_CUDA_TRY(cudaSetDevice(h.device));
    cudaDeviceProp prop;
    GBG_CUDA_TRY(cudaGetDeviceProperties(&prop, h.device));
    int bucket = 1;
    while (bucket < h.max_samples) bucket <<= 1;
    char key[512];
    std::snprintf(key, sizeof(key), "%s|n=%d|S<=%d|f32", prop.name, h.n, bucket);
    std::map<std::string, int> cache;
    const int nv = gbg::population_variant_count(h.n);
    if (cache_path) {
        cache = read_tune_cache(cache_path);
        auto it = cache.find(key);
        if (it != cache.end() && it->second >= 0 && it->second < nv) {
            h.pop_variant = it->second;
            *chosen = it->second;
            return GBG_OK;
        }
    }
    // probe: samples near the centre, about 24 steps each, from an initial
    // Gaussian wide enough (sigma = n / 4) to be nonzero on every tissue cell,
    // so that the skipping kernel visits every live tile of every round, as it
    // does once a population's tumours have spread
    std::vector<gbg_sample> probe(probe_samples);
    const double L = h.n * 0.1, c = 0.5 * (h.n - 1);
    for (int i = 0; i < probe_samples; ++i) {
        const double Dw = 0.0013;
        double dt, Dwu, Dgu, r = 0.05;
        gbg::reference_dt(h.n, Dw, L, false, &dt, &Dwu, &Dgu, &r);
        probe[i] = gbg_sample{Dw, 0.05, c + (i % 3) - 1.0, c, c + (i % 5) - 2.0, 23.5 * dt};
    }
    gbg_batch_opts o{L, 0.1, 0.25 * h.n, 0, 0.0};
    int best = 0;
    float best_ms = 1e30f;
    const int saved = h.pop_variant;
    for (int v = 0; v < nv; ++v) {
        h.pop_variant = v;
        float ms = 0.f;
        for (int rep = 0; rep < 2; ++rep) {
            int rc = gbg_batch_solve(hh, probe.data(), probe_samples, &o, nullptr, nullptr, nullptr);
            if (rc) {
                h.pop_variant = saved;
                return rc;
            }
            rc = gbg_last_population_ms(hh, &ms);
            if (rc) {
                h.pop_variant = saved;
                return rc;
            }
        }
        if (ms < best_ms) {
            best_ms = ms;
            best = v;
        }
    }
    h.pop_variant = best;
    *chosen = best;
    if (cache_path) {
        cache[key] = best;
        write_tune_cache(cache_path, cache);
    }
    return GBG_OK;
}

int gbg_sync(gbg_handle *hh) {
    if (int rc = check_handle(hh)) return rc;
    GBG_CUDA_TRY(cudaSetDevice(hh->h.device));
    GBG_CUDA_TRY(cudaStreamSynchronize(hh->h.stream));
    return GBG_OK;
}

}  // extern "C"
