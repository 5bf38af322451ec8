/*
 * sp_oracle.h — TEST INFRASTRUCTURE.  CPU restatement ("oracle") of the
 * SpatialPy engine hot path, used only by tests/, the smoke check and the
 * CPU-baseline leg of bench.py.  It is never linked into libspgpu.so.
 *
 * NSM semantics follow nsm_core__take_step (src/simulate_rdme.cpp:211-472)
 * and the NRM queue contract (src/NRMConstant_v5.cpp): per-voxel next-event
 * times, fresh exponential draws for every voxel an event touches, events
 * in increasing time.  Propensities, selection scans and waiting times are
 * single precision with a fixed operation order; the clock is double.  The random streams are Philox4x32-10 (Salmon et al.,
 * SC'11) keyed by the trajectory seed, so the GPU engine can be checked
 * against this file event for event; against the reference's own
 * mt19937_64 streams the comparison is statistical.
 *
 * Parity status: pinned.  The neighbour sets, dWdr and D_ij match the compiled
 * reference (oracle/_ref, built by build_ref.sh) element-wise; the NSM
 * ensembles match reference ensembles statistically (tests/golden/).
 */
#ifndef SP_ORACLE_H
#define SP_ORACLE_H
#include <stdint.h>
#include "../include/spgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Philox4x32-10 block: out = philox(ctr, key) */
void spo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* -log(u) for u in (0,1), evaluated with a fixed operation order */
double spo_neglog(double u);

/* Neighbour lists (particle.cpp:150-210, kd_fix_rad_search.cpp:160-176):
 * ascending r^2, ties by index; kmax per particle.  Positions `xq` are query
 * points, `xt` the searched points (pass the same array for a static search).
 * Returns 0, or -1 if a list overflows kmax. */
int spo_neighbors(int32_t n, int32_t dim, const double *xq, const double *xt, double h,
                  const double *mass, const double *rho, int32_t kmax, int32_t *count,
                  int32_t *idx, double *dist, double *dwdr, double *dij);

/* Ddiag[i*S+s] and cumulative weights cdf[(i*S+s)*kmax + k] from the lists
 * (simulate_rdme.cpp:131-152 and the destination scan :353-367), summed in
 * double and rounded to float. */
void spo_diffusion_tables(const sp_scenario *sc, int32_t kmax, const int32_t *count,
                          const int32_t *idx, const double *dij, float *ddiag, float *cdf);
/* single-precision -log(u), the variate of the NSM waiting times */
float spo_neglog_f(float u);

/*
 * Run one NSM trajectory on a static domain.
 * out: [num_outputs][N][S] counts (may be NULL); ev: (reactions, diffusions).
 * Returns SP_TRAJ_* status.
 */
int spo_nsm_trajectory(const sp_scenario *sc, const uint32_t *u0, uint64_t seed, int32_t selection,
                       int32_t *out, int64_t *ev);

/* Ensemble over `ntraj` seeds with `threads` POSIX threads (0 = all cores).
 * out: [ntraj][num_outputs][N][S] or NULL; ev: [ntraj*2]. */
int spo_nsm_ensemble(const sp_scenario *sc, const uint32_t *u0, const uint64_t *seeds,
                     int32_t ntraj, int32_t selection, int32_t threads, int32_t *out,
                     int64_t *ev, int32_t *status);

/* SDPD flow (sdpd_oracle.c), FP64 and FP32 builds.  mode bits:
 *   1 = Gauss-Seidel density reads in the boundary-volume-fraction pass (the
 *       order a single engine thread produces, model.cpp:284-288)
 *   2 = neighbour distances between moved query and start-of-step points (the
 *       kd-tree is built once per step, simulate_threads.cpp:80-108)
 *   4 = with 2: a particle's distance to its own start-of-step point is the
 *       predictor displacement |dt vt| (the FP32 engine's rule)
 * State arrays are [N*3] / [N] in double; nsteps engine steps from step0. */
/* Neighbour lists of the last step's force pass (count[N], idx/dij[N*kmax]),
 * D_ij (particle.cpp:181-187) computed in the build's arithmetic from the
 * post-predictor densities, widened to double. */
typedef struct spo_sdpd_lists {
    int32_t *count;
    int32_t *idx;
    double *dij;
} spo_sdpd_lists;
/* chem: deterministic concentrations C and fluxes Q ([N*S] double each) to
 * advance with the flow when sc->enable_pde (NULL: none); nu: the particle
 * viscosities [N], updated by boundary conditions (NULL: sc->nu). */
typedef struct spo_chem {
    double *C;
    double *Q;
    double *nu;
} spo_chem;
/* The FP32 flow's stored state between calls (ignored by spo_sdpd_f64):
 * positions as float pairs hi + lo [N*3] each, densities as float deviations
 * from rho0 [N].  valid = 0 on the first call (state taken from x and rho);
 * every call writes it back and sets valid = 1.  NULL: taken from x and rho
 * on every call (exact only for a single call). */
typedef struct spo_f32_state {
    float *xh;
    float *xl;
    float *drho;
    int32_t valid;
} spo_f32_state;
int spo_sdpd_f64(const sp_scenario *sc, int32_t step0, int32_t nsteps, int32_t mode, int32_t kmax,
                 double *x, double *v, double *vt, double *rho, double *F, double *Fbp,
                 double *Frho, int32_t *nbr_count, spo_sdpd_lists *lists, spo_chem *chem,
                 spo_f32_state *fs);
int spo_sdpd_f32(const sp_scenario *sc, int32_t step0, int32_t nsteps, int32_t mode, int32_t kmax,
                 double *x, double *v, double *vt, double *rho, double *F, double *Fbp,
                 double *Frho, int32_t *nbr_count, spo_sdpd_lists *lists, spo_chem *chem,
                 spo_f32_state *fs);

/* Deterministic chemistry (Model.enable_pde; model.cpp:151-189,
 * simulate.cpp:81-88, 166-171) with the layouts the matrices are written in
 * (species-major diffusion, N[s][r]).
 * spo_chem_half: C += Q dt/2 (not when first), the boundary conditions on
 * concentrations (positions [N*pstride]), then Q = 0 when clear_q.
 * spo_chem_flux: Q from neighbour lists (skipping r = 0 and r > h) and the
 * reactions' ODE rate programs at time t.
 * spo_chem_static: a static domain from C = u0 over the time span, with the
 * oracle's fixed neighbour lists; out [num_outputs][N][S]. */
void spo_chem_half(const sp_scenario *sc, double *C, double *Q, const double *pos, int pstride,
                   int first, int clear_q);
void spo_chem_flux(const sp_scenario *sc, const double *C, double *Q, const int32_t *cnt,
                   const int32_t *idx, const double *dist, const double *dwdr, int kstride,
                   const double *mass, const double *rho, double t);
int spo_chem_static(const sp_scenario *sc, const uint32_t *u0, int32_t kmax, double *out);
/* boundary conditions on v, nu, rho of particle i at position p (after the
 * predictor and after the corrector, simulate.cpp:88, 171) */
void spo_flow_bcs(const sp_scenario *sc, int i, const double p[3], double v[3], double *nu,
                  double *rho);

/*
 * Moving domain with stochastic species (simulate_threads.cpp:232-281 with
 * simulate_rdme.cpp:53-68 on a non-static domain): every step runs the SDPD
 * step (precision 32 or 64, `mode` bits as above), rebuilds Ddiag and the
 * destination weights from that step's lists, the volumes m/rho from the
 * end-of-step density, and every trajectory's event queue at t = step*dt
 * (Philox build stream index = step), then runs that trajectory's events up
 * to (step+1)*dt.  The SDPD step runs on one thread, the trajectories of a
 * step on `threads` POSIX threads (0 = all cores).
 * out: [ntraj][num_outputs][N][S] counts or NULL; px/prho:
 * [num_outputs][N*3] / [num_outputs][N] flow state or NULL; ev: [ntraj*2];
 * status: [ntraj]; chem_out: [num_outputs][N][S] deterministic
 * concentrations (enable_pde) or NULL.  Returns 0, -1 on a list overflow,
 * 2 on NaN state.
 */
int spo_coupled_ensemble(const sp_scenario *sc, const uint32_t *u0, const uint64_t *seeds,
                         int32_t ntraj, int32_t selection, int32_t precision, int32_t mode,
                         int32_t kmax, int32_t threads, int32_t *out, int64_t *ev,
                         int32_t *status, double *px, double *prho, double *chem_out);

#ifdef __cplusplus
}
#endif
#endif
