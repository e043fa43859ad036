/* gbglioma -- GB300-native Fisher-Kolmogorov tumour-growth step and imaging
 * log-likelihood for GliomaUQ, behind a plain C ABI.
 *
 * Conventions
 *  - Every function returns int status: GBG_OK (0) or a negative GBG_ERR_*.
 *    gbg_last_error() gives a one-line message for the calling thread's last
 *    failure.
 *  - Fields are cubic grids of n^3 cells, x fastest: cell (x, y, z) is at
 *    x + n*(y + n*z) -- the order of Matrix::D3D (source/Glioma/Matrix.h:593-602).
 *    The domain is the unit cube, periodic in x, y and z
 *    (source/MRAGcore/MRAGrid.inl:37-39), cell size h = 1/n.
 *  - Host pointers unless a name ends in _device. The caller owns host arrays;
 *    the library owns its device memory.
 *  - A handle owns one CUDA stream. A handle is not thread-safe; different
 *    handles may be used from different threads at once.
 *  - There is no CPU fallback: without a usable GPU, gbg_create fails.
 */
#ifndef GBGLIOMA_H
#define GBGLIOMA_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBG_VERSION_MAJOR 0
#define GBG_VERSION_MINOR 1

enum gbg_status {
    GBG_OK = 0,
    GBG_ERR_ARG = -1,         /* bad argument (null pointer, size, range) */
    GBG_ERR_CUDA = -2,        /* a CUDA runtime call failed */
    GBG_ERR_TIMEOUT = -3,     /* a bounded device-side wait ran out */
    GBG_ERR_NONFINITE = -4,   /* NaN/Inf in an input that must be finite */
    GBG_ERR_STATE = -5,       /* call out of order (e.g. step before anatomy) */
    GBG_ERR_NOMEM = -6,       /* device allocation failed */
    GBG_ERR_UNSUPPORTED = -7  /* configuration not supported by this build */
};

/* Arithmetic of the step.
 *  GBG_PREC_F64    : the reference built with -D_MRAG_REAL_=double: double
 *                    storage and arithmetic, every operation rounded as the
 *                    reference's source writes it (bit-identical results).
 *  GBG_PREC_F32REF : the reference's default build (Real=float,
 *                    source/MRAGcore/MRAGCommon.h:43-48): float storage and
 *                    Dw/Dg/rho, double per-cell temporaries, dphidt rounded to
 *                    float (bit-identical results).
 *  GBG_PREC_F32    : fast path: float storage and float arithmetic with the
 *                    face diffusivities precomputed; its error against the
 *                    FP64 result is measured and stated, not zero. */
enum gbg_precision { GBG_PREC_F64 = 0, GBG_PREC_F32REF = 1, GBG_PREC_F32 = 2 };

typedef struct gbg_handle gbg_handle;

typedef struct {
    int n;           /* cells per side (n >= 4) */
    int precision;   /* enum gbg_precision */
    int device;      /* CUDA device ordinal */
    int max_samples; /* capacity of the batched population (0: no batch buffers) */
} gbg_config;

/* ---- lifetime ------------------------------------------------------------ */
int gbg_create(const gbg_config *cfg, gbg_handle **out);
int gbg_destroy(gbg_handle *h);
const char *gbg_last_error(void);
int gbg_version(int *major, int *minor);

/* ---- anatomy and state ----------------------------------------------------
 * gbg_set_anatomy replaces the p_w/p_g fields of every cell (the block fields
 * of CCell_extended, source/Glioma/Glioma_Types.h:27-28) and invalidates the
 * precomputed face diffusivities. Values must be finite. */
int gbg_set_anatomy(gbg_handle *h, const double *p_w, const double *p_g);
/* density field phi (CCell_extended::phi), n^3 doubles, converted to the
 * storage type (rounded to float in the float modes). */
int gbg_set_phi(gbg_handle *h, const double *phi);
int gbg_get_phi(gbg_handle *h, double *phi);

/* ---- the step ---------------------------------------------------------------
 * nsteps fused steps of Glioma_ReactionDiffusionOperator<3> (Case2 branch,
 * source/Glioma/Glioma_ReactionDiffusionOperator.h:148-218) followed by
 * UpdateTumor<3> (:254-261), on the uniform periodic grid. Replaces one call of
 * Glioma_HG_UQ::_reactionDiffusionStep (source/Glioma/Glioma_HG_UQ.cpp:266-277),
 * i.e. BlockProcessing::pipeline_process(rhs) + BlockProcessing::process(update)
 * per step. Dw, Dg are the operator's arguments (already divided by L^2), rho
 * in 1/day, dt in days. In the float modes Dw, Dg and rho are rounded to float
 * as the reference's Real-typed operator members are. */
int gbg_rd_step(gbg_handle *h, double Dw, double Dg, double rho, double dt, long nsteps);

/* The whole time loop of Glioma_HG_UQ::run for a uniform grid
 * (source/Glioma/Glioma_HG_UQ.cpp:519-552): Dw_file in cm^2/day and rho in 1/day
 * as read from HGG_InputParameters.txt, tend in days, L the brain length in cm
 * (Glioma_HG_UQ.cpp:104). Computes Dw = Dw_file/L^2, Dg = 0.1*Dw,
 * dt = 0.99*h^2/(6*max(Dw,Dg)) with the reference's rounding, then steps while
 * t <= tend. Writes the step count and dt if the pointers are non-null. */
int gbg_run(gbg_handle *h, double Dw_file, double rho, double tend, double L, long *nsteps_out,
            double *dt_out);

/* ---- the MALA variant (exact modes) ------------------------------------------
 * Glioma_HG_UQ_MALA carries two more cell fields, the slopes sRho = dphi/drho
 * and sD = dphi/dDw (CCell_extended::sRho, sD,
 * source/Glioma/Glioma_Types.h:61-62), zero at the start.
 *
 * gbg_set_slopes: n^3 doubles each, converted to the storage type; NULL sets
 * that field to zero. gbg_get_slopes reads both back. GBG_PREC_F64 and
 * GBG_PREC_F32REF only (GBG_ERR_UNSUPPORTED otherwise). */
int gbg_set_slopes(gbg_handle *h, const double *sRho, const double *sD);
int gbg_get_slopes(gbg_handle *h, double *sRho, double *sD);

/* nsteps steps of Glioma_HG_UQ_MALA::_reactionDiffusionMALAStep
 * (source/Glioma/Glioma_HG_UQ_MALA.cpp:575-591): the RD right-hand side and
 * the slopes' right-hand side (Glioma_MALAslopesRHS<3>,
 * source/Glioma/Glioma_MALA_SlopesOperator.h:13-188) from the state before
 * the step, then UpdateTumor and UpdateMALAslopes (:190-226). Arguments as
 * gbg_rd_step. The slopes operator is the reference's as written: its
 * tissue tensor is the non-Case2 harmonic mean with Neumann doubling, and
 * its sources are phi (1 - phi) and div(T grad phi) without the linearised
 * reaction term, so sRho and sD are the reference's slopes, not exact
 * derivatives of phi (gbg_adjoint gives those). Slopes not set are zero. */
int gbg_mala_step(gbg_handle *h, double Dw, double Dg, double rho, double dt, long nsteps);

/* The MALA variant's whole loop (Glioma_HG_UQ_MALA::run,
 * source/Glioma/Glioma_HG_UQ_MALA.cpp:717-758): arguments, parameter rescale,
 * step rule and loop as gbg_run. */
int gbg_run_mala(gbg_handle *h, double Dw_file, double rho, double tend, double L, long *nsteps_out,
                 double *dt_out);

/* ---- imaging log-likelihood (source/Likelihood/source/HGG_Likelihood.cpp) --
 * Observations: PET, T1, T2 fields (n^3 doubles each, PET_data.dat,
 * T1_data.dat, T2_data.dat) and the Sphere.dat point set, npoints x 3 voxel
 * indices stored column-major as Matrix::D2D stores them (all x, then all y,
 * then all z). selective!=0 evaluates the T1/T2 terms on those points
 * (HGG_Likelihood.cpp:105-124), otherwise on every voxel (:97-104). */
typedef struct {
    double pet_sigma2, pet_scale, t1_uc, t2_uc, slope; /* LikelihoodInput.txt order */
    int step_pet, step_ti, selective;                  /* -stepPet, -stepTi, -selectivePoints */
} gbg_lik_params;

typedef struct {
    double l_pet, l_t1, l_t2; /* the three partial log-likelihoods */
    double total;             /* log L = l_pet + l_t1 + l_t2; Likelihood.txt holds -total */
    long n_pet;               /* PET voxels used */
} gbg_lik_result;

int gbg_set_observations(gbg_handle *h, const double *pet, const double *t1, const double *t2,
                         const double *points, long npoints, const gbg_lik_params *p);
/* log-likelihood of the handle's current phi (HGG_Likelihood::run, :173-189),
 * accumulated in double. */
int gbg_loglik(gbg_handle *h, gbg_lik_result *out);

/* ---- batched population ----------------------------------------------------
 * S independent forward solves sharing the handle's anatomy, each from a
 * Gaussian initial density phi0 = peak*exp(-|x-x0|^2/(2 sigma^2)) (voxel
 * units) on tissue cells, each with its own parameters and step count (the
 * reference's time loop per sample), followed by each sample's
 * log-likelihood against the handle's observations. The unit of work of the
 * external sampler's one `brain` + `likelihood` process pair per sample. */
typedef struct {
    double Dw;   /* cm^2/day, as in HGG_InputParameters.txt */
    double rho;  /* 1/day */
    double x0, y0, z0; /* seed, voxel units (cell centre of voxel i is i) */
    double tend; /* days */
} gbg_sample;

typedef struct {
    double L;          /* brain length in cm (n*0.1 for 1 mm voxels) */
    double ic_peak;    /* initial peak density */
    double ic_sigma;   /* initial width in voxels */
    int with_loglik;   /* evaluate the likelihood per sample */
    double dt0;        /* time grid. 0: the reference's time loop per sample
                          (dt from Dw, steps while t <= tend). Otherwise a
                          smooth grid of gbg_adjoint_grad (see there): the
                          densities and log L equal its forward model bit for
                          bit (GBG_PREC_F32 state). */
} gbg_batch_opts;

/* Host entry: copies the S samples in, solves, copies loglik (S results, may
 * be null when with_loglik==0) and per-sample step counts (may be null) out.
 * phi_out, if non-null, receives S*n^3 floats of final densities. Float
 * modes only (GBG_PREC_F32 or GBG_PREC_F32REF). */
int gbg_batch_solve(gbg_handle *h, const gbg_sample *samples, int S, const gbg_batch_opts *o,
                    gbg_lik_result *loglik, long *nsteps_out, float *phi_out);
/* gbg_batch_solve runs as one CUDA graph launch per call: the first call
 * with a given S and options captures the device-side sequence (schedule,
 * sort, initial densities, the persistent cooperative population kernel,
 * the likelihood reduction) from the handle's stream, later calls copy the
 * samples in, replay the graph and copy the results out. Graphs are kept per
 * population-kernel shape (gbg_set_population_variant, gbg_autotune), at most
 * 8 per handle, and captured anew after the anatomy or the observations
 * change. enabled = 0 launches the kernels one by one
 * instead (the same results, bit for bit). Default: enabled. */
int gbg_set_batch_graphs(gbg_handle *h, int enabled);
/* Device-resident entry: samples_device (S gbg_sample) and loglik_device (S
 * gbg_lik_result, or null) are device pointers; runs on the handle's stream
 * and returns without synchronising. */
int gbg_batch_solve_device(gbg_handle *h, const gbg_sample *samples_device, int S,
                           const gbg_batch_opts *o, gbg_lik_result *loglik_device);

/* ---- posterior propagation statistics -------------------------------------------
 * Per-cell mean and variance of S density fields as the reference's
 * propagation tool computes them over the posterior samples' HGG_data.dat
 * files (Glioma_HG_Propagation::_ic_PatientCasePropagation,
 * source/Glioma/Glioma_HG_Propagation.cpp:346-440, PropagationStatistics,
 * Glioma_PropagationStatisticsOperator.h:24-50) in its default Real = float:
 * the sum in sample order, the squared deviations from (1/S) * sum, both
 * scaled by 1/S. reference_rules != 0 keeps the tool's index rule: cells with
 * a zero x, y or z index get mean = var = 0 (it accumulates mapped indices in
 * (0, size] only). Device pointers; fields_device holds S fields of n^3 floats
 * (x fastest) one after another; the call enqueues on stream (a
 * cudaStream_t, null = legacy default) and allocates nothing. */
int gbg_field_statistics(int n, const float *fields_device, int S, int reference_rules, float *mean_device,
                         float *var_device, void *stream);
/* The batched solve of the S samples (as gbg_batch_solve; S <= max_samples),
 * then the statistics above over their final densities, written to the host
 * arrays mean and var (n^3 each). */
int gbg_batch_statistics(gbg_handle *h, const gbg_sample *samples, int S, const gbg_batch_opts *o,
                         int reference_rules, double *mean, double *var);

/* ---- gradients for MALA: discrete adjoint ----------------------------------------
 * No reference counterpart for the adjoint itself; the forward model it
 * differentiates is the fast-path step on a smooth time grid: a step dt,
 * n = ceil(tend/dt) steps, the last one shortened to end exactly at tend
 * (the reference's integer step count makes its output piecewise constant
 * in Dw and tend). dt0 > 0: dt = dt0 for every sample (fixed grid; dt0 must
 * satisfy the stability limit of the largest Dw and rho,
 * 0.99 h^2 / (6 Dw_max / L^2 + rho_max h^2 / 2)).
 * dt0 < 0: dt = |dt0| * 0.99 h^2 / (6 Dw / L^2 + rho h^2 / 2) per sample
 * (scaled grid, stable for |dt0| <= 1): the reference's step rule
 * 0.99 h^2 / (6 Dw / L^2) bounds only the diffusion part of the explicit
 * step; with it, wherever the density is near 1 in white matter the
 * checkerboard mode grows by |1 - 12 a - b| > 1 per step (a = dt Dw / (L h)^2,
 * b = dt rho), the clamp to [0, 1] bounds the oscillation and the final
 * density amplifies rounding differences (a 1e-10 change of the initial state
 * reached 4e-3 relative L2 after 399 steps at 128^3). The added rho term makes
 * 12 a + b = 1.98 |dt0|, so that mode decays. The discrete model keeps the
 * continuous model's symmetry (Dw, rho, tend) -> (c Dw, c rho, tend / c),
 * under which the density at tend is unchanged. Gradients
 * are of the log-likelihood (gbg_set_observations) with respect to
 * (Dw, rho, x0, y0, z0, tend), in the units of gbg_sample, written as
 * grad[6*s + 0..5]; loglik[s] receives log L of the same forward model
 * (either pointer may be null; with grad null no adjoint sweep runs).
 * States are checkpointed every checkpoint_every steps (<= 0: about
 * sqrt(steps), which minimises the stored states) and each segment is
 * recomputed for its backward sweep; state_precision is GBG_PREC_F32 (float
 * states) or GBG_PREC_F64 (double states). Works on any handle made by
 * gbg_create; the working set (checkpoints, one segment of states, adjoint
 * fields) is kept by the handle between calls and grows when a call needs
 * more, until gbg_destroy. */
typedef struct {
    double dt0;            /* > 0: fixed step in days; < 0: scaled grid (-1: the stable step) */
    int checkpoint_every;
    double L;              /* brain length in cm */
    double ic_peak, ic_sigma;
    int state_precision;   /* GBG_PREC_F32 or GBG_PREC_F64 */
} gbg_adjoint_opts;

int gbg_adjoint_grad(gbg_handle *h, const gbg_sample *samples, int S, const gbg_adjoint_opts *o,
                     double *loglik, double *grad);

/* ---- affine density model (tangent screening) ------------------------------------
 * No reference counterpart. phi(delta) = m * clamp(phi0 + sum_p delta_p J_p, 0, 1)
 * with m the fast path's tissue mask and 1 <= P <= 16 basis fields:
 * gbg_affine_set copies phi0 (n^3 floats) and J (P x n^3 floats, field-
 * major; e.g. J_p = d phi / d u_p at the reference sample in the sampler's
 * coordinates u, plus second-order fields); gbg_affine_loglik writes log L
 * (the handle's observations) of B models given by their coefficients delta
 * (B x P doubles; e.g. u - u_ref and products of its components). The cheap first stage
 * of delayed-acceptance MCMC around a posterior mode. GBG_PREC_F32 handles;
 * the handle keeps the fields until gbg_destroy. The models are evaluated at
 * the observation lists' cells only (phi0, J and m gathered there once per
 * model and observation set), with the same float operations as forming the
 * whole field, so log L equals that of the formed field bit for bit. */
int gbg_affine_set(gbg_handle *h, int P, const float *phi0, const float *J);
int gbg_affine_loglik(gbg_handle *h, int B, const double *delta, gbg_lik_result *out);

/* The screening chain on the GPU: `steps` Metropolis steps on
 *   log pi*(v) = log L(affine model at c(v - u_ref)) + log prior(v)
 * for B chains in one launch (the first stage of delayed-acceptance MCMC).
 * v are the sampler's coordinates; u = Ai v, theta_i = exp(u_i) where bit i of
 * log_mask is set (else u_i); the prior is uniform on lo <= theta <= hi with
 * the seed voxel rint(theta_2..4) inside the mask set by
 * gbg_affine_set_prior_mask (n^3 bytes, x fastest), as a density in v (log
 * prior = sum of the log coordinates' u_i). c(d) = d, or with quad_axis = a
 * (d, d_a^2 / 2, d_a d_i for i != a) -- the model needs 6 or 12 fields. A step
 * is, with probability axis_prob, a redraw of coordinate `axis` from its
 * prior conditional (accepted with the likelihood ratio); with probability
 * ind_prob an independence proposal ind_mean + ind_chol xi for the other
 * coordinates (accepted with the Metropolis-Hastings ratio of that Gaussian;
 * ind_inv = ind_chol^-1, with `axis` decoupled in both); otherwise
 * v + step * chol xi on the other coordinates (matrices row-major 6 x 6).
 * v (B x 6) is updated in place; lp_start / lp_end get log pi* at the chains'
 * start and end points (-inf outside the prior); counts (B x 6, may be null)
 * random-walk accepts and steps, redraw accepts and redraws, independence
 * accepts and proposals. seed fixes the random numbers (counter-based). No
 * reference counterpart. */
typedef struct {
    int axis;          /* coordinate redrawn from its prior conditional, -1: none */
    double axis_prob;  /* probability of a redraw per step */
    double step;       /* random-walk scale */
    double chol[36];   /* random-walk factor */
    double u_ref[6];   /* the affine model's centre */
    int quad_axis;     /* second-order terms along this coordinate, -1: none */
    double Ai[36];     /* u = Ai v */
    int log_mask;      /* bit i: theta_i = exp(u_i) */
    double lo[6], hi[6];
    double ind_prob;       /* probability of an independence move per step */
    double ind_mean[6], ind_chol[36], ind_inv[36];
} gbg_affine_chain_opts;
int gbg_affine_set_prior_mask(gbg_handle *h, const unsigned char *mask);
/* entries of the observation lists gbg_set_observations built: PET voxels and
 * T1/T2 points */
int gbg_observation_counts(gbg_handle *h, long *n_pet, long *n_ti);
int gbg_affine_chain(gbg_handle *h, const gbg_affine_chain_opts *o, int B, int steps, unsigned long long seed,
                     double *v, double *lp_start, double *lp_end, int *counts);

/* ---- learned surrogate (delayed-acceptance screening) ----------------------------
 * No reference counterpart. A small 3D convolutional U-Net maps a sample's
 * parameters (as input channels: the anatomy, a blob at the seed, the
 * rescaled Dw, rho and tend, and the distance to a Fisher-KPP front of radius
 * 2 sqrt(D rho) tend) to its final density on a grid `factor` (= 2) times
 * coarser than the handle's. It is trained by the library's own bf16
 * tensor-core kernels (forward and backward) on densities that the handle's
 * batched solver computes for the given training samples, with Adam on fp32
 * master weights. gbg_surrogate_loglik predicts densities (upsampled to the
 * solver grid, zero off tissue) and evaluates the handle's likelihood on
 * them: the cheap first stage of delayed-acceptance MCMC, whose second stage
 * is the solver. The handle must be GBG_PREC_F32 with max_samples >= 1 and
 * n a multiple of 8; gbg_surrogate_create copies its anatomy. */
typedef struct gbg_surrogate gbg_surrogate;
typedef struct {
    int factor;      /* solver grid / surrogate grid, 2 */
    int batch_max;   /* largest batch of train/loss_grad/loglik */
    double L;        /* brain length in cm */
    double dw_lo, dw_hi, rho_lo, rho_hi, t_lo, t_hi; /* prior ranges for input scaling */
    unsigned long long seed; /* initial weights */
} gbg_surrogate_config;

int gbg_surrogate_create(gbg_handle *h, const gbg_surrogate_config *cfg, gbg_surrogate **out);
int gbg_surrogate_destroy(gbg_surrogate *s);
int gbg_surrogate_nparams(gbg_surrogate *s, long *count);
int gbg_surrogate_get_params(gbg_surrogate *s, float *params);
int gbg_surrogate_set_params(gbg_surrogate *s, const float *params);
/* trains on S samples for `epochs` passes; *loss = mean loss of the last pass */
int gbg_surrogate_train(gbg_surrogate *s, const gbg_sample *samples, int S, int epochs, int batch,
                        double lr, unsigned long long seed, double *loss);
/* loss and flat parameter gradient of one batch against host targets on the
 * surrogate grid (B fields of (n/2)^3 floats); grad may be null */
int gbg_surrogate_loss_grad(gbg_surrogate *s, const gbg_sample *samples, int B, const float *targets,
                            double *loss, float *grad);
/* the network's input channels of B samples, B x (n/2)^3 x 16 floats */
int gbg_surrogate_features(gbg_surrogate *s, const gbg_sample *samples, int B, float *out);
/* predicted log-likelihoods of B samples (host); phi, if non-null, receives
 * the B predicted densities on the solver grid */
int gbg_surrogate_loglik(gbg_surrogate *s, const gbg_sample *samples, int B, gbg_lik_result *out,
                         float *phi);
/* the kernels of the forward and data-gradient convolutions: 0 = mma.sync
 * (m16n8k16 bf16 tiles in registers), 1 = tcgen05 (128 x Cout tiles,
 * accumulator in tensor memory, operands in shared memory). The weight
 * gradient always runs on mma.sync. Default 1. */
int gbg_surrogate_set_engine(gbg_surrogate *s, int engine);

/* ---- multiresolution block grid ----------------------------------------------
 * MRAG's grid of 16^3 blocks at mixed levels (source/MRAGcore/MRAGrid.h:44-186):
 * block b at level l covers [index/2^l, (index+1)/2^l) of the unit cube with
 * h = 1/(2^l * 16). Fields are block-major, 4096 cells per block, x fastest
 * inside a block. Ghost cells come from MRAG's ghost instruction tables
 * (BoundaryInfoBlock, source/MRAGcore/MRAGBoundaryBlockInfo.h:69-176) flattened:
 * ghost g of block b (g in [0, 1736), the order BlockLab::load visits the 26
 * neighbour regions for the stencil [-1, 2), source/MRAGcore/MRAGBlockLab.h:256-295)
 * is sum_k value(src_block[k], src_cell[k]) * w[k] over
 * k in [start[b*1736+g], start[b*1736+g+1]), evaluated in the handle's Real
 * type in that order; w[k] is the Real product of the entry's three weights.
 * src_block indexes the blocks in the order given to gbg_amr_set_grid. */
typedef struct {
    int level, ix, iy, iz;
} gbg_block;

typedef struct {
    int max_blocks;  /* capacity */
    int precision;   /* GBG_PREC_F64 or GBG_PREC_F32REF */
    int device;
} gbg_amr_config;

int gbg_amr_create(const gbg_amr_config *cfg, gbg_handle **out);
int gbg_amr_set_grid(gbg_handle *h, int nblocks, const gbg_block *blocks, const double *p_w,
                     const double *p_g, const double *phi);
int gbg_amr_set_ghosts(gbg_handle *h, const long *start, const int *src_block, const int *src_cell,
                       const double *w, long nentries);
/* nsteps steps of the RD operator + UpdateTumor on every block, exactly as
 * BlockProcessing::pipeline_process(rhs) + process(update) do on the MRAG
 * grid (source/Glioma/Glioma_HG_UQ.cpp:266-277). */
int gbg_amr_step(gbg_handle *h, double Dw, double Dg, double rho, double dt, long nsteps);
/* GBG_PREC_F32 block grids: the form of the step, both with the same
 * results bit for bit. 0 (default): ghosts evaluated while each block's lab
 * is filled, face coefficients stored once per face; 1: a separate ghost
 * pass and per-cell tables (kept for comparison). */
int gbg_amr_fast_variant(gbg_handle *h, int variant);
int gbg_amr_get_phi(gbg_handle *h, double *phi);
/* per block: the largest interpolating-wavelet detail magnitude of phi,
 * BlockFWT::multichannel_fwt + FWTReport::getOverAll_DetailMaxMag
 * (source/MRAGcore/MRAGBlockFWT.h:184-190,219-298,447-468) -- the quantity
 * Science::AutomaticRefinement/Compression compare with their tolerances. */
int gbg_amr_fwt_detail(gbg_handle *h, double *detail);
/* Regrid data movement: build a new set of blocks from the current grid.
 * New block i is kind[i] = GBG_REMAP_COPY of current block src[8i]; or
 * GBG_REMAP_SPLIT, the child src[8i+1] (x + 2y + 4z) of current block src[8i]
 * by interpolating-wavelet prediction (BlockSplitter::_splitBlocks,
 * source/MRAGcore/MRAGBlockSplitter.h:24-100, using the current ghost
 * tables); or GBG_REMAP_COLLAPSE of the eight current blocks src[8i..8i+7]
 * (child x + 2y + 4z) by decimation (BlockCollapser::_collapseBlocks,
 * source/MRAGcore/MRAGBlockCollapser.h:19-61). phi, p_w and p_g all move.
 * The ghost tables of the new grid must be set before the next step. */
#define GBG_REMAP_COPY 0
#define GBG_REMAP_SPLIT 1
#define GBG_REMAP_COLLAPSE 2
int gbg_amr_remap(gbg_handle *h, int nblocks_new, const gbg_block *blocks_new, const int *kind,
                  const int *src);
/* phi on the uniform grid of gpd^3 cells, hf = 1/gpd, as
 * Glioma_HG_UQ::_dumpUQoutput writes HGG_data.dat (Glioma_HG_UQ.cpp:309-372).
 * reference_rules != 0 replicates a block cell r^3 times with r = 1, 2, 3 for
 * h = hf, 2 hf, 3 hf and r = 4 otherwise, as the reference does (so blocks
 * coarser than 4 hf leave cells unwritten: they are 0 here); reference_rules
 * == 0 replicates h/hf exactly. Blocks finer than hf contribute the cells on
 * the dump grid's points. */
int gbg_amr_dump_uniform(gbg_handle *h, int gpd, int reference_rules, double *out);

/* ---- adaptive grid: ghost tables, regrid plans, the adaptive time loop -------
 * Host-only (no GPU, no handle): the ghost instruction tables of a periodic
 * block tree, as MRAG_BBInfoCreator::createBoundaryInfoBlock and
 * Grid::getBoundaryInfo build them (source/MRAGcore/MRAG_BBInfoCreator.inl:902-1316,
 * MRAGrid.inl:514-700) for Interpolating 2nd-order wavelets and the stencil
 * [-1, 2), in the layout gbg_amr_set_ghosts takes: start[nb*1736 + 1]
 * offsets and nentries (source block, source cell, weight) entries. With
 * src_block, src_cell or w null only start and *nentries are written (a size
 * query); otherwise capacity must be at least *nentries. The blocks must tile
 * the unit cube as the leaves of a block tree. */
int gbg_amr_ghost_tables(int nblocks, const gbg_block *blocks, long *start, int *src_block, int *src_cell,
                         double *w, long capacity, long *nentries);
/* Host-only. Grid::refine's plan for the flagged blocks (flagged[i] != 0):
 * Refiner_SpaceExtension::createPlan + Refiner::createPlan
 * (source/MRAGscience/MRAGRefiner_SpaceExtension.h:25-67, MRAGcore/MRAGRefiner.h:45-195,
 * level jump 1, periodic): also every block with a finer neighbour that is
 * not a periodic image, never a block on max_level (< 0: no limit), and
 * every block the level-jump rule then requires. Writes the new blocks with
 * the gbg_amr_remap kind/src arrays (8 src entries per block) for them,
 * *nb_new and the number of refined blocks. */
int gbg_amr_plan_refine(int nblocks, const gbg_block *blocks, const unsigned char *flagged, int max_level,
                        int capacity, gbg_block *blocks_new, int *kind, int *src, int *nb_new, int *nrefined);
/* Host-only. Grid::compress's plan (Compressor::createPlan,
 * source/MRAGcore/MRAGCompressor.h:68-144, level jump 1, periodic): eight
 * siblings collapse when all are flagged and all their neighbours are within
 * one level of the parent. Output as gbg_amr_plan_refine. */
int gbg_amr_plan_compress(int nblocks, const gbg_block *blocks, const unsigned char *flagged, int capacity,
                          gbg_block *blocks_new, int *kind, int *src, int *nb_new, int *ncollapsed);
/* Compiles and installs the ghost tables of the handle's current blocks
 * (replaces gbg_amr_set_ghosts for grids the library manages). */
int gbg_amr_build_ghosts(gbg_handle *h);
/* Science::AutomaticRefinement with one pass (source/MRAGscience/MRAGScienceCore.h:42-108):
 * the blocks below max_level whose FWT detail is >= tol are refined by the
 * plan above, the data moved on the device and the new tables installed. */
int gbg_amr_auto_refine(gbg_handle *h, double tol, int max_level, int *nrefined);
/* Science::AutomaticCompression (MRAGScienceCore.h:117-177): passes of FWT,
 * flag (detail < tol), collapse, new tables, until a pass collapses nothing; a
 * block not flagged in a pass is not examined again in the call. */
int gbg_amr_auto_compress(gbg_handle *h, double tol, int *ncollapsed);
/* The current blocks, in the device order (capacity >= the block count;
 * blocks null: only *nblocks). */
int gbg_amr_get_blocks(gbg_handle *h, gbg_block *blocks, int capacity, int *nblocks);

typedef struct {
    double Dw_file;      /* cm^2/day, as HGG_InputParameters.txt gives it */
    double rho;          /* 1/day */
    double tend;         /* days */
    double L;            /* brain length in cm */
    double dumpfreq;     /* a regrid whenever t passes the next multiple (-dumpfreq) */
    int bpd;             /* blocks per dimension of the initial grid: dt from h = 1/(16 bpd) */
    int adaptive;        /* regrid at the dump times (-adaptive 1) */
    int max_level;       /* finest level a refinement may create (_MAXLEVEL_) */
    int final_refine;    /* the refinement after the loop (Glioma_HG_UQ.cpp:574-575) */
    double refine_tol;   /* 1e-4 in the reference (Glioma_Types.h:462) */
    double compress_tol; /* 1e-5 (Glioma_Types.h:463) */
} gbg_amr_run_opts;
/* Glioma_HG_UQ::run (source/Glioma/Glioma_HG_UQ.cpp:511-582) on the handle's
 * grid: Dw /= L^2, Dg = 0.1 Dw (rounded to float in GBG_PREC_F32REF, as the
 * default build's Real), dt = 0.99 h^2 / (6 max(Dw, Dg)), steps while
 * t <= tend, the automatic regrids at the dump times and after the loop when
 * adaptive. Ghost tables are compiled by the library. Writes the step and
 * regrid counts. */
int gbg_amr_run(gbg_handle *h, const gbg_amr_run_opts *opts, long *steps, int *regrids);
/* No reference counterpart. Statistics of the handle's latest gbg_amr_run:
 * cell-steps computed (blocks x 4096 summed over the steps), the wall time
 * of the steps and of the regrids (each regrid waits for the steps before
 * it, then FWT on the device, plans and ghost tables on the host, data
 * movement on the device), the number of regrid calls, and the fewest and
 * most blocks the grid had. */
typedef struct {
    long long cell_steps;
    double step_seconds, regrid_seconds;
    int regrid_calls, min_blocks, max_blocks;
} gbg_amr_run_stats;
int gbg_amr_last_run_stats(gbg_handle *h, gbg_amr_run_stats *stats);

/* ---- synthetic observations -----------------------------------------------------
 * PET, T1 and T2 observations from a tumour density as the reference's
 * synthetic-data program makes them (brain -anatomy syntheticData,
 * Glioma_ProcessSyntheticData.cpp:61-104 and 107-221, run :406-430) in its
 * float Real: PET = u where u >= uc_t2, T1 = [u >= uc_t1], T2 = [u >= uc_t2];
 * PET normalised by its maximum; noise alpha * N(0, 1) from drand48 pairs
 * through Box-Muller on the cells with PET > 0, a pair drawn at every cell
 * visited while the count of noised cells is even; normalised again; the
 * centre of mass (unit cube, float sums in loop order) of the noised PET
 * (what the program writes to HGG_TumorIC.bin). The loops visit the blocks
 * of the uniform 16^3-block grid in `order` (nblocks = (n/16)^3 blocks of
 * gbg_block; the reference's order comes from MRAG's node map, ordered by
 * node address) or, with order null, x fastest; cells x fastest inside a
 * block. tumor, pet, t1, t2: n^3 doubles, x fastest (HGG_data.dat and the
 * PET/T1/T2_data.dat contents); n = 16 * 2^l. The program's values are
 * uc_t1 = 0.8, uc_t2 = 0.3, alpha = 0.02 and the unseeded drand48 state (0
 * with glibc). Fails with GBG_ERR_ARG when no cell reaches uc_t2 (the
 * program divides by a zero maximum). */
typedef struct {
    double uc_t1, uc_t2;   /* T1 / T2 thresholds */
    double alpha;          /* noise standard deviation (0: none) */
    unsigned long long seed48;  /* drand48 state before the first draw */
} gbg_synthetic_opts;
int gbg_synthetic_observations(int n, const double *tumor, int nblocks, const gbg_block *order,
                               const gbg_synthetic_opts *o, double *pet, double *t1, double *t2,
                               float *centre_of_mass);

/* ---- introspection ---------------------------------------------------------- */
/* number of kernels this handle has launched since creation */
int gbg_launch_count(gbg_handle *h, long long *count);
/* the handle's CUDA stream (a cudaStream_t) */
int gbg_stream(gbg_handle *h, void **stream);
/* synchronise the handle's stream */
int gbg_sync(gbg_handle *h);
/* device time in milliseconds of the handle's most recent population-kernel
 * launch (the persistent step kernel of gbg_batch_solve* and of the fast
 * single solve), measured with CUDA events around that launch on the handle's
 * stream; waits for it to finish. */
int gbg_last_population_ms(gbg_handle *h, float *ms);
/* No reference counterpart. Cell-steps the most recent population-kernel
 * launch computed: the tiles it visited times the cells of a tile. The
 * skipping kernel (the batched solver's default) visits only the tiles whose
 * output can be nonzero, so this is at most the population's step count times
 * n^3; the dense register kernel visits every tile of every active sample.
 * Waits for the launch to finish; GBG_ERR_UNSUPPORTED for the other kernel
 * families, which do not count. */
int gbg_last_population_cells(gbg_handle *h, long long *cell_steps);

/* ---- population-kernel shape and autotuner --------------------------------
 * No counterpart in the reference (its TBB pipeline has a compile-time
 * thread hint). The fast population kernel has several tile shapes per grid
 * size (rows per tile x samples per CTA). gbg_population_variants reports
 * how many; gbg_set_population_variant picks one by index (0 = default).
 * gbg_autotune times every shape on a probe population of probe_samples
 * samples (<= max_samples) over the handle's anatomy and keeps the fastest;
 * with cache_path non-null it first looks the choice up in that JSON file,
 * keyed by GPU name, n, population-size bucket and precision, and records
 * new choices there. Writes the chosen index to *chosen. GBG_PREC_F32 only. */
int gbg_population_variants(gbg_handle *h, int *count);
int gbg_set_population_variant(gbg_handle *h, int index);
int gbg_population_variant_shape(gbg_handle *h, int index, int *rows, int *samples_per_cta,
                                 int *threads);
/* The kernel a variant launches, with its template arguments and tile depth
 * (e.g. "k_population8<32,4> TZ 16"), as a NUL-terminated string of at most
 * len bytes. */
int gbg_population_variant_name(gbg_handle *h, int index, char *buf, int len);
int gbg_autotune(gbg_handle *h, int probe_samples, const char *cache_path, int *chosen);

/* ---- log-likelihood without any allocation -----------------------------------
 * No counterpart in the reference: an addition for callers that cannot
 * allocate device memory -- a host framework whose device memory is owned by
 * its own allocator, or a real-time loop with a fixed memory budget. It evaluates the
 * same log-likelihood as gbg_loglik for one density field, without a handle,
 * and calls no cudaMalloc, cudaFree or other allocating routine.
 *
 * The caller passes everything in device memory: the field phi_device (n^3
 * floats, x fastest) and the compact observation lists that
 * gbg_set_observations builds internally --
 *   pet_idx/pet_val  : cell index and PET value of every voxel with
 *                      ix,iy,iz = 0 mod stepPet and PET > 0 (n_pet entries)
 *   ti_idx/t1_val/t2_val : cell index and T1/T2 value of every evaluation
 *                      point (n_ti entries)
 * -- the scalar parameters in p (its step/selective fields are not used: the
 * lists already encode them), and out_device, one gbg_lik_result. n must be
 * the field's edge and every index in pet_idx and ti_idx must lie in
 * [0, n^3): the kernels read phi_device at those indices unchecked.
 * stream is a cudaStream_t (null: the legacy default stream); the call only
 * enqueues work and does not synchronise.
 *
 * Its scratch is a fixed device array inside the library (3 doubles per chunk
 * of 2048 list entries, at most GBG_NOALLOC_MAX_ENTRIES entries, 96 KiB),
 * which every GPU that loads the library keeps until the process exits. The
 * first call in a CUDA context (the primary context of a device, a context
 * the caller made current with the driver API, or the new primary context
 * after cudaDeviceReset) looks that array's address up with the context
 * current. Every call
 * shares the array: calls whose kernels may overlap on the GPU (different
 * streams, or different host threads) race and must be serialised by the
 * caller. Lists longer than the maximum are rejected with GBG_ERR_ARG. */
#define GBG_NOALLOC_MAX_ENTRIES (4096L * 2048L)
int gbg_loglik_noalloc(const float *phi_device, int n, const int *pet_idx, const double *pet_val,
                       long n_pet, const int *ti_idx, const double *t1_val, const double *t2_val,
                       long n_ti, const gbg_lik_params *p, gbg_lik_result *out_device,
                       void *stream);

#ifdef __cplusplus
}
#endif
#endif
