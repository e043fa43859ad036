/* CPU oracle for the GliomaUQ hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's arithmetic, used by tests/ as the
 * checker, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg. The
 * product (gliomauq_gb300/, include/) never links or calls it.
 *
 * Parity of this restatement is pinned against the reference itself, compiled
 * in place by oracle/Makefile into oracle/_ref/ (tests/golden/ holds the
 * fixtures those binaries produced, and tests/golden/make_golden.py the script).
 *
 * Fields are x-fastest: cell (x,y,z) of an n^3 grid is at x + n*(y + n*z).
 * The grid is periodic in x, y and z (source/MRAGcore/MRAGrid.inl:37-39).
 */
#ifndef GLIOMAUQ_ORACLE_H
#define GLIOMAUQ_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One explicit-Euler step of Glioma_ReactionDiffusionOperator<3> (Case2) +
 * UpdateTumor<3> on a uniform periodic n^3 grid, double storage (the reference
 * built with -D_MRAG_REAL_=double). phi_out must not alias phi_in.
 * Follows source/Glioma/Glioma_ReactionDiffusionOperator.h:148-218 (RHS) and
 * :254-261 (update). nthreads<=0 uses all online cores. */
void orc_rd_step_f64(int n, const double *pw, const double *pg, const double *phi_in,
                     double *phi_out, double Dw, double Dg, double rho, double dt, double h,
                     int nthreads);

/* Same step with the reference's default build semantics: float storage
 * (Real=float, source/MRAGcore/MRAGCommon.h:43-48), float Dw/Dg/rho, double
 * per-cell temporaries, dphidt rounded to float before the update. */
void orc_rd_step_f32ref(int n, const float *pw, const float *pg, const float *phi_in,
                        float *phi_out, float Dw, float Dg, float rho, double dt, double h,
                        int nthreads);

/* nsteps steps of the above, ping-ponging through an internal buffer; the
 * result is left in phi (in place). */
void orc_rd_solve_f64(int n, const double *pw, const double *pg, double *phi, double Dw,
                      double Dg, double rho, double dt, double h, long nsteps, int nthreads);
void orc_rd_solve_f32ref(int n, const float *pw, const float *pg, float *phi, float Dw,
                         float Dg, float rho, double dt, double h, long nsteps, int nthreads);

/* The reference's CPU structure restated for timing (the "port" CPU
 * baseline): 16^3 blocks of 41-float array-of-structs cells, a per-block
 * (16+2)^3 lab filled from the block and its periodic neighbours
 * (BlockLab::load, source/MRAGcore/MRAGBlockLab.h:154-301), the operator
 * writing dphidt into the block, then a separate update pass
 * (Glioma_HG_UQ::_reactionDiffusionStep, source/Glioma/Glioma_HG_UQ.cpp:266-277),
 * with blocks handed to worker threads dynamically as the TBB pipeline does.
 * Arithmetic is identical to orc_rd_step_f32ref. n must be a multiple of 16. */
typedef struct orc_blockgrid orc_blockgrid;
orc_blockgrid *orc_blockgrid_create(int n, const float *pw, const float *pg, const float *phi);
void orc_blockgrid_steps(orc_blockgrid *g, float Dw, float Dg, float rho, double dt, double h,
                         long nsteps, int nthreads);
void orc_blockgrid_get_phi(const orc_blockgrid *g, float *phi);
void orc_blockgrid_destroy(orc_blockgrid *g);

/* HGG_Likelihood (source/Likelihood/source/HGG_Likelihood.cpp):
 *   PET term  :40-75, T1/T2 terms :77-128, Bernoulli :136-153, sgn :155-160.
 * model/pet/t1/t2 are n^3 double fields. points is the Sphere.dat matrix
 * (D2D<double> npoints x 3, stored column-major: all x, then all y, then z);
 * selective!=0 uses it, otherwise all voxels. Results are the three
 * long-double partial log-likelihoods widened to what the platform's long
 * double is, returned as double, plus the PET voxel count. */
typedef struct {
    double pet_sigma2, pet_scale, t1_uc, t2_uc, slope;
} orc_lik_params;
typedef struct {
    double l_pet, l_t1, l_t2, total; /* total = l_pet + l_t1 + l_t2 (log L) */
    long n_pet;
} orc_lik_result;
void orc_loglik(int nx, int ny, int nz, const double *model, const double *pet,
                const double *t1, const double *t2, const double *points, long npoints,
                const orc_lik_params *p, int step_pet, int step_ti, int selective,
                orc_lik_result *out);

/* One step of the MALA variant (Glioma_HG_UQ_MALA::_reactionDiffusionMALAStep,
 * source/Glioma/Glioma_HG_UQ_MALA.cpp:575-591): the RD step above plus the
 * slopes sRho = dphi/drho and sD = dphi/dDw of Glioma_MALAslopesRHS<3> and
 * UpdateMALAslopes<3> (source/Glioma/Glioma_MALA_SlopesOperator.h:122-187,
 * 215-223), both right-hand sides from the state before the step. The
 * slopes' tissue tensor is the non-Case2 one (harmonic means of
 * p_w + p_g Dg/Dw, Neumann doubling where a face is 0) and their sources are
 * phi (1 - phi) and div(T grad phi), as the reference writes them. Outputs
 * must not alias inputs. f64: double storage; f32ref: the default build
 * (float storage, double fluxes, rates rounded to float). */
void orc_mala_step_f64(int n, const double *pw, const double *pg, const double *phi_in,
                       const double *sr_in, const double *sd_in, double *phi_out,
                       double *sr_out, double *sd_out, double Dw, double Dg, double rho,
                       double dt, double h);
void orc_mala_step_f32ref(int n, const float *pw, const float *pg, const float *phi_in,
                          const float *sr_in, const float *sd_in, float *phi_out, float *sr_out,
                          float *sd_out, float Dw, float Dg, float rho, double dt, double h);

/* Number of steps the reference's time loop takes: while (t <= tend) t += dt
 * (source/Glioma/Glioma_HG_UQ.cpp:544-552). */
long orc_num_steps(double dt, double tend);

#ifdef __cplusplus
}
#endif
#endif
