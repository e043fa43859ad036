// Internal declarations shared by the libgbglioma translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/gbglioma.h"

namespace gbg {

// Thread-local last error message (gbg_last_error).
void set_error(const std::string &msg);

#define GBG_CUDA_TRY(expr)                                                            \
    do {                                                                              \
        cudaError_t _e = (expr);                                                      \
        if (_e != cudaSuccess) {                                                      \
            ::gbg::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));     \
            return _e == cudaErrorMemoryAllocation ? GBG_ERR_NOMEM : GBG_ERR_CUDA;    \
        }                                                                             \
    } while (0)

// Device-side error codes written to the handle's status word.
// DEV_DRAIN_TIMEOUT: after a copy timeout, waiting for the copies still in
// flight timed out as well (they may have landed after the CTA left).
enum DeviceStatus : int {
    DEV_OK = 0,
    DEV_BARRIER_TIMEOUT = 1,
    DEV_COPY_TIMEOUT = 2,
    DEV_MMA_TIMEOUT = 3,
    DEV_DRAIN_TIMEOUT = 4
};

// Compact observation lists for the likelihood (see likelihood.cu).
struct ObsDevice {
    int n_pet = 0;           // PET voxels kept (stride and PET > 0)
    int *pet_idx = nullptr;  // cell indices
    double *pet_val = nullptr;
    int n_ti = 0;            // T1/T2 evaluation points
    int *ti_idx = nullptr;
    double *t1_val = nullptr;
    double *t2_val = nullptr;
    double pet_sigma2 = 0, pet_scale = 0, t1_uc = 0, t2_uc = 0, slope = 0;
    bool valid = false;
};

// Multiresolution block grid state (amr.cu)
struct AmrState {
    int max_blocks = 0, nb = 0, cur = 0;
    void *phi[2] = {nullptr, nullptr};
    void *pw = nullptr, *pg = nullptr, *b0 = nullptr;
    void *gphi = nullptr, *gpw = nullptr, *gpg = nullptr;  // ghost values
    double *df = nullptr;      // six face diffusivities per cell
    int *level = nullptr;      // per block
    long *gstart = nullptr;    // ghost-table offsets, nb*1736+1
    int *gsrc_block = nullptr, *gsrc_cell = nullptr;
    double *gw = nullptr;
    // fast FP32 mode: the tables in 32-bit form for the fused step (offsets,
    // source cell as block * 4096 + cell, float weights)
    int *gstart32 = nullptr, *gsrc32 = nullptr;
    float *gw32 = nullptr;
    int fast_variant = 0;      // 0: fused ghosts, per-face tables; 1: separate ghost pass
    double *detail = nullptr;  // FWT maxima per block
    void *pw2 = nullptr, *pg2 = nullptr;  // remap targets
    int *bidx = nullptr;       // block index (ix, iy, iz) per block
    int *rkind = nullptr, *rsrc = nullptr;  // remap plan
    bool ghosts_valid = false, tables_valid = false;
    double tab_Dw = -1, tab_Dg = -1;
    std::vector<gbg_block> hblocks;  // host copy of the blocks, in the device order
    gbg_amr_run_stats last_run{};    // statistics of the latest gbg_amr_run
};

struct BatchGraph {
    int S = 0, with_loglik = 0, variant = 0;
    double L = 0, ic_peak = 0, ic_sigma = 0, dt0 = 0;
    const void *samples = nullptr, *lik = nullptr;  // device pointers the graph reads / writes
    unsigned long long gen = 0, last_use = 0;
    long long launches = 0;  // kernels per replay
    long long tile_cells = 0;  // the captured population kernel's cells per tile
    cudaGraphExec_t exec = nullptr;
};

struct Handle {
    int n = 0;
    size_t N = 0;
    int prec = GBG_PREC_F64;
    int device = 0;
    int max_samples = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    long long launches = 0;

    // anatomy, kept in double so any mode can rebuild its tables
    double *pw = nullptr, *pg = nullptr;
    bool anatomy_set = false;

    // single-solve state: phi ping-pong in the storage type
    void *phi[2] = {nullptr, nullptr};
    int cur = 0;
    bool phi_set = false;

    // exact modes: brain sum b0 (storage type) and face diffusivities (double)
    void *b0 = nullptr;
    double *dfx = nullptr, *dfy = nullptr, *dfz = nullptr;
    double tab_Dw = -1, tab_Dg = -1;  // (Dw, Dg) the tables were built for
    bool tables_valid = false;

    // MALA variant (exact modes): slopes sRho, sD ping-pong in the storage
    // type (index cur, with phi), and the slopes' tissue tensor, 6 doubles per
    // cell (SoA, faces W, E, S, N, B, F) for the ratio Dg/Dw it was built for
    void *sr[2] = {nullptr, nullptr}, *sd[2] = {nullptr, nullptr};
    bool slopes_set = false;
    double *mala_tt = nullptr;
    double mala_ratio = -1;
    bool mala_valid = false;

    // fast mode: unit-diffusivity face coefficients and tissue mask (float SoA)
    float *cx = nullptr, *cy = nullptr, *cz = nullptr, *msk = nullptr;
    float *cxs = nullptr;  // cx with the sign bit set where msk is 0 (population kernels)
    double fast_ratio = -1;  // Dg/Dw the fast coefficients were built for
    bool fast_valid = false;

    // batched population buffers
    float *bphi[2] = {nullptr, nullptr};  // max_samples * N each
    void *bwork = nullptr;                // per-sample schedule records
    size_t bwork_bytes = 0;
    int *dev_status = nullptr;            // device status word
    unsigned *barrier = nullptr;          // grid barrier {count, generation}, then a
                                          // 64-bit visited-tile counter
    long long pop_tile_cells = 0;         // cells per tile of the latest launch (0: not counted)

    // population-kernel shape (index into the candidates for this n; 0 = default)
    int pop_variant = 0;

    // CUDA graphs of the batched solve (gbg_batch_solve): one per sample
    // count, options and population-kernel shape, captured from the handle's
    // stream. state_gen counts the changes that invalidate a captured graph
    // (a buffer it names reallocated, a table or tile list it reads rebuilt,
    // new observations); a graph captured at another generation is captured
    // anew.
    unsigned long long state_gen = 0;
    unsigned long long graph_clock = 0;  // replay counter (least recently used graph)
    bool batch_graphs = true;
    std::vector<BatchGraph> graphs;

    // tiles of the skipping population kernel (k_population10): a tile (RY
    // rows of full x-rows by TZ planes) is live when one of its cells has a
    // mask of 1; live_list holds the live tile indices (count in *live_count,
    // device); built for tile depth live_tz from the fast tables' mask
    unsigned char *tile_live = nullptr;
    int *live_list = nullptr;
    int *live_count = nullptr;
    int live_tz = 0, live_ry = 0;
    bool live_valid = false;

    // events bracketing the latest population-kernel launch
    cudaEvent_t ev_pop[2] = {nullptr, nullptr};
    bool ev_pop_recorded = false;

    // multiresolution grid (handles made by gbg_amr_create)
    bool is_amr = false;
    AmrState amr;

    // likelihood
    ObsDevice obs;
    double *lik_partials = nullptr;  // scratch for the two-pass reduction
    size_t lik_partials_cap = 0;
    void *lik_out = nullptr;         // device gbg_lik_result scratch
    int lik_out_cap = 0;

    // adjoint working set, grow-only
    void *adj_ws = nullptr;
    size_t adj_ws_bytes = 0;

    // affine density model phi0 + sum_p delta_p J_p (gbg_affine_*); aff_cols
    // holds phi0, the P basis fields and the tissue mask gathered at the
    // observation lists' cells (rebuilt when the model or the observations
    // change)
    float *aff_phi0 = nullptr, *aff_J = nullptr, *aff_cols = nullptr;
    int aff_P = 0;
    size_t aff_cols_cap = 0;  // floats
    bool aff_cols_stale = true;
    double *aff_delta = nullptr;
    size_t aff_delta_cap = 0;  // doubles
    unsigned char *aff_mask = nullptr;  // the prior's seed-voxel mask (n^3, affine chain)
    float4 *aff_rec = nullptr;          // per observation point: model + value, 16 floats (affine chain)
    size_t aff_rec_cap = 0;             // points
    void *aff_chain = nullptr;          // affine chain scratch, grow-only
    size_t aff_chain_bytes = 0;
};

// ---- rd_exact.cu ----
int exact_build_tables(Handle &h, double Dw, double Dg);
int exact_steps(Handle &h, double Dw, double Dg, double rho, double dt, long nsteps);
// nsteps steps of the MALA variant: phi (exact_steps) and the slopes; the
// slopes must be allocated and set
int mala_steps(Handle &h, double Dw, double Dg, double rho, double dt, long nsteps);

// ---- rd_fast.cu ----
// Per-sample schedule record of the batched solver (stored sorted by nsteps,
// longest first, for the population kernel; unsorted for everything else).
struct SampleRec {
    float a, b;   // dt*Dw/h^2 and dt*rho
    int nsteps;   // step count
    int order;    // sample index
    double dt;
    float a2, b2; // coefficients of the last step (== a, b on the reference schedule)
};
// Layout of Handle::bwork, each region 256-byte aligned, cap = max(1, max_samples):
// unsorted records | sorted records | rank_of ints | staged gbg_sample inputs |
// initial-support boxes (4 ints per sample, unsorted order; see k_gaussian_ic).
inline size_t bwork_align(size_t b) { return (b + 255) & ~(size_t)255; }
inline int bwork_cap(const Handle &h) { return h.max_samples > 1 ? h.max_samples : 1; }
inline size_t bwork_off_sorted(const Handle &h) { return bwork_align(bwork_cap(h) * sizeof(SampleRec)); }
inline size_t bwork_off_rank(const Handle &h) { return 2 * bwork_off_sorted(h); }
inline size_t bwork_off_samples(const Handle &h) {
    return bwork_off_rank(h) + bwork_align(bwork_cap(h) * sizeof(int));
}
inline size_t bwork_off_boxes(const Handle &h) {
    return bwork_off_samples(h) + bwork_align(bwork_cap(h) * sizeof(gbg_sample));
}
inline size_t bwork_total(const Handle &h) { return bwork_off_boxes(h) + bwork_align(bwork_cap(h) * 4 * sizeof(int)); }
inline SampleRec *batch_unsorted(Handle &h) { return reinterpret_cast<SampleRec *>(h.bwork); }
inline SampleRec *batch_sorted(Handle &h) {
    return reinterpret_cast<SampleRec *>((char *)h.bwork + bwork_off_sorted(h));
}
inline int *batch_rank_of(Handle &h) { return reinterpret_cast<int *>((char *)h.bwork + bwork_off_rank(h)); }
inline gbg_sample *batch_samples(Handle &h) {
    return reinterpret_cast<gbg_sample *>((char *)h.bwork + bwork_off_samples(h));
}
inline int *batch_boxes(Handle &h) { return reinterpret_cast<int *>((char *)h.bwork + bwork_off_boxes(h)); }
int fast_build_tables(Handle &h, double ratio);
// smooth time grid (fixed dt0, last step shortened): per-sample records into
// dev_out (S entries, unsorted order)
int launch_schedule_smooth(Handle &h, const gbg_sample *samples_device, int S, double L, double dt0,
                           SampleRec *dev_out);
// Gaussian initial densities of S samples (float fields, the batched solver's IC)
// Population-kernel steps on S float states starting in buf0 (buf1 the
// second buffer, S x N each): sample s (record s, order = s) takes
// recs[s].nsteps steps with coefficients a, b, the last one a2, b2, and ends
// in buffer (nsteps & 1). recs: S device records; sorted / rank: device
// scratch for S records / ints. Dense kernels only (no temporal blocking, no
// skipping: the states may be anything). slot > 0 keeps every state instead:
// step k reads buf0 + k * slot and writes buf0 + (k + 1) * slot (buf1 unused).
// box non-null: the skipping kernel may run, given per-sample support boxes
// as launch_gaussian_ic records them (indexed by record order) of an initial
// state whose support lies within them grown by grow0 cells; with slot 0 it
// also needs that state zero on every cell without the mask unless
// grow0 = 0, and a zero-filled buf1 (in slot mode it writes every tile).
int population_steps(Handle &h, float *buf0, float *buf1, const SampleRec *recs, SampleRec *sorted, int *rank,
                     int S, size_t slot = 0, const int *box = nullptr, int grow0 = 0);
bool population_supported(int n);
// Builds and allocates what batch_solve_device would build or allocate on
// first use (fast tables, the skipping kernel's tile list, likelihood
// partials for S samples), so that a stream capture of it records launches
// and copies only.
int batch_prepare(Handle &h, int S, const gbg_batch_opts &o);
int lik_reserve(Handle &h, int S);
// batch_solve_device through a CUDA graph of it (captured on first use for
// this S and options, replayed after); no step counts.
int batch_graph_run(Handle &h, const gbg_sample *samples_device, int S, const gbg_batch_opts &o,
                    gbg_lik_result *loglik_device);
void batch_graphs_clear(Handle &h);
int launch_gaussian_ic(Handle &h, const gbg_sample *samples_device, int S, double peak, double sigma,
                       float *phi, int *box = nullptr);
int fast_steps_single(Handle &h, double Dw, double rho, double dt, long nsteps);
int population_variant_count(int n);
int population_variant_shape(int n, int vi, int *ry, int *g, int *threads);
int population_variant_name(int n, int vi, char *buf, int len);
// reads and clears the device status word (synchronises the stream)
int check_device_status(Handle &h);
int batch_solve_device(Handle &h, const gbg_sample *samples_device, int S,
                       const gbg_batch_opts &o, gbg_lik_result *loglik_device, long *nsteps_host);

// ---- propagation.cu ----
// batched solve of S samples, then per-cell mean and variance of their final
// densities into mean_device / var_device (n^3 floats each)
int batch_statistics(Handle &h, const gbg_sample *samples_device, int S, const gbg_batch_opts &o,
                     int reference_rules, float *mean_device, float *var_device);

// ---- amr.cu ----
int amr_region_start(int code);
int amr_alloc(Handle &h);
void amr_free(Handle &h);
int amr_set_grid(Handle &h, int nb, const gbg_block *blocks, const double *pw, const double *pg,
                 const double *phi);
int amr_set_ghosts(Handle &h, const long *start, const int *src_block, const int *src_cell, const double *w,
                   long nentries);
int amr_steps(Handle &h, double Dw, double Dg, double rho, double dt, long nsteps);
int amr_get_phi(Handle &h, double *phi);
int amr_fwt_detail(Handle &h, double *detail);
int amr_remap(Handle &h, int nbn, const gbg_block *blocks, const int *kind, const int *src);
int amr_dump_uniform(Handle &h, int gpd, int reference_rules, double *out);
// ---- amr_plan.cu ----
// ghost tables of the handle's blocks, compiled on the host and installed
int amr_build_ghosts(Handle &h);
// Science::AutomaticRefinement with one pass / AutomaticCompression to a fixpoint
int amr_auto_refine(Handle &h, double tol, int max_level, int *refined);
int amr_auto_compress(Handle &h, double tol, int *collapsed);
int amr_run(Handle &h, const gbg_amr_run_opts &o, long *steps, int *regrids);

// ---- adjoint.cu ----
int adjoint_grad(Handle &h, const gbg_sample *samples, int S, const gbg_adjoint_opts &o, double *loglik,
                 double *grad);

// ---- surrogate.cu ----
struct Surrogate;
int surrogate_create(Handle &h, const gbg_surrogate_config &c, Surrogate **out);
void surrogate_destroy(Surrogate *s);
long surrogate_nparams(const Surrogate &s);
int surrogate_batch_max(const Surrogate &s);
int surrogate_set_engine(Surrogate &s, int engine);
const float *surrogate_prediction(const Surrogate &s);  // last predicted densities, solver grid
int surrogate_get_params(Surrogate &s, float *out);
int surrogate_set_params(Surrogate &s, const float *in);
int surrogate_loss_grad(Surrogate &s, const gbg_sample *samples, int B, const float *targets_host, double *loss,
                        float *grad_host);
int surrogate_features(Surrogate &s, const gbg_sample *samples, int B, float *out);
int surrogate_train(Surrogate &s, const gbg_sample *samples, int S, int epochs, int batch, double lr,
                    unsigned long long seed, double *loss_out);
int surrogate_predict(Surrogate &s, const gbg_sample *samples_device, int B, gbg_lik_result *lik_device);

// ---- likelihood.cu ----
int lik_set_observations(Handle &h, const double *pet, const double *t1, const double *t2,
                         const double *points, long npoints, const gbg_lik_params &p);
// phi_f32 or phi_f64 (one non-null): S fields of N cells at stride N.
int lik_evaluate(Handle &h, const float *phi_f32, const double *phi_f64, int S,
                 gbg_lik_result *out_device);
// population: sample s's final field is in buf[recs[s].nsteps & 1] + s*N.
// log L of B affine models evaluated at the observation cells only
// (delta_device: B x P; cols: likelihood.cu's AffineSource layout)
int lik_evaluate_affine(Handle &h, const float *cols, int P, const double *delta_device, int B,
                        gbg_lik_result *out_device);
int lik_evaluate_population(Handle &h, const float *buf0, const float *buf1,
                            const SampleRec *recs_unsorted, int S, gbg_lik_result *out_device);

// dt and unit-cube Dw/Dg as Glioma_HG_UQ::run computes them (float modes round
// Dw and Dg to float at each assignment).
void reference_dt(int n, double Dw_file, double L, bool f32, double *dt, double *Dw, double *Dg,
                  double *rho_in_out);
long reference_num_steps(double dt, double tend);

// ---- affine.cu ----
int affine_set(Handle &h, int P, const float *phi0, const float *J);
int affine_loglik(Handle &h, int B, const double *delta_host, gbg_lik_result *lik_device);
// phi0, J and the mask gathered at the observation lists' cells (aff_cols)
int affine_gather_columns(Handle &h);
// ---- affine_chain.cu ----
int affine_set_prior_mask(Handle &h, const unsigned char *mask);
int affine_chain(Handle &h, const gbg_affine_chain_opts &o, int B, int steps, unsigned long long seed,
                 double *v, double *lp_start, double *lp_end, int *counts);

}  // namespace gbg

struct gbg_handle {
    gbg::Handle h;
};
