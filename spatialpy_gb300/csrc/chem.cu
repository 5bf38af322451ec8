// chem.cu — deterministic chemistry (Model.enable_pde): concentrations C
// that start at u0, with fluxes Q from SPH diffusion between neighbours and
// from the reactions' ODE propensities (model.cpp:151-189), advanced by two
// half steps per engine step (simulate.cpp:81-85 after the predictor,
// simulate.cpp:166-169 after the corrector), with the boundary conditions
// that target a concentration applied after each half step.
//
// Per step, three launches:
//   chem_half(step > 0)  C += Q dt/2, boundary conditions, Q = 0
//   chem_flux            Q from the step's neighbour lists and C
//   chem_half            C += Q dt/2, boundary conditions
// State C, Q: [N][S] double, one copy per model instance (it is the same for
// every trajectory).
//
// The reference indexes its diffusion matrix type-major here and its dense
// stoichiometry as [reaction][species] (model.cpp:165, 186), which reads out
// of bounds whenever the species and reaction counts differ; this file uses
// the layouts the matrices are written in (species-major diffusion
// solver.py:269-286, N[s][r] solver.py:225-231).  Compiled with -fmad=false.
#include <cuda_runtime.h>

#include <cstdint>

#include "chem.cuh"
#include "common.cuh"
#include "nsm_prog.cuh"

namespace spg {

// boundary conditions on concentrations, in order (boundarycondition.py:121-167)
__device__ __forceinline__ void chem_bcs(const ChemDev& D, int i, double px, double py,
                                         double pz, double* c) {
    for (int b = 0; b < D.nbc; b++) {
        const int tg = D.bc_target[b];
        if (tg < SP_BC_C) continue;
        const double* bx = D.bc_box + 6 * b;
        if (px >= bx[0] && px <= bx[1] && py >= bx[2] && py <= bx[3] && pz >= bx[4] &&
            pz <= bx[5] && (D.bc_type[b] == 0 || D.bc_type[b] == D.type[i]))
            c[tg - SP_BC_C] = D.bc_value[3 * b];
    }
}

template <typename PT>
__global__ void chem_half(ChemDev D, const PT* pos, int pstride, double coef, int clear_q) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= D.N) return;
    double* c = D.C + (size_t)i * D.S;
    double* q = D.Q + (size_t)i * D.S;
    if (coef != 0.0)
        for (int s = 0; s < D.S; s++) c[s] = c[s] + q[s] * coef;
    if (D.nbc) {
        const PT* p = pos + (size_t)i * pstride;
        chem_bcs(D, i, (double)p[0], (double)p[1], (double)p[2], c);
    }
    if (clear_q)
        for (int s = 0; s < D.S; s++) q[s] = 0.0;
}

// Q of particle i: SPH diffusion over its neighbours (skipping r = 0 and
// r > h, model.cpp:90-95) in list order, then each reaction's ODE rate times
// its stoichiometry.  LT: type of the list distances and dWdr and of the
// particle masses and densities (double for static lists and the FP64 flow,
// float for the FP32 flow).
template <typename LT>
__global__ void chem_flux(ChemDev D, const int* cnt, const int* idx, const LT* dist,
                          const LT* dwdr, int kstride, const LT* mass, const LT* rho, double t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= D.N) return;
    const int S = D.S;
    const double h = D.h;
    const double* ci = D.C + (size_t)i * S;
    double* q = D.Q + (size_t)i * S;
    const double mi = (double)mass[i], ri = (double)rho[i];
    const int ti = D.type[i];
    const int m = cnt[i];
    for (int k = 0; k < m; k++) {
        const size_t o = (size_t)i * kstride + k;
        const double r = (double)dist[o];
        if (r / h > 1.0 || r == 0.0) continue;
        const int j = idx[o];
        const double mj = (double)mass[j], rj = (double)rho[j];
        const double wfd = (1.0 / (r + 0.001 * h)) * (double)dwdr[o];
        const double base = 2.0 * ((mi * mj) / (mi + mj)) * ((ri + rj) / (ri * rj)) * (r * r) *
                            wfd / ((r * r) + 0.01 * h * h);   // Tartakovsky et al. 2007
        const double* cj = D.C + (size_t)j * S;
        for (int s = 0; s < S; s++)
            q[s] = q[s] + D.diffusion[s * D.T + (ti - 1)] * (ci[s] - cj[s]) * base;
    }
    const double vol = mi / ri;
    for (int r = 0; r < D.R; r++) {
        if (D.allowed && !D.allowed[r * (D.T + 1) + ti]) continue;
        auto xs = [&](int s) { return ci[s]; };
        const double flux = run_program(D.code + D.code_off[r], D.consts, D.data, D.N, i, xs,
                                        vol, t, ti);
        for (int s = 0; s < S; s++) q[s] = q[s] + (double)D.stoich[s * D.R + r] * flux;
    }
}

void chem_launch_half(const ChemDev& D, const double* pos, bool first, bool clear_q,
                      cudaStream_t st) {
    const int tb = 256;
    chem_half<double><<<(D.N + tb - 1) / tb, tb, 0, st>>>(D, pos, 3, first ? 0.0 : 0.5 * D.dt,
                                                          clear_q ? 1 : 0);
}

void chem_launch_half4f(const ChemDev& D, const float* pos4, bool first, bool clear_q,
                        cudaStream_t st) {
    const int tb = 256;
    chem_half<float><<<(D.N + tb - 1) / tb, tb, 0, st>>>(D, pos4, 4, first ? 0.0 : 0.5 * D.dt,
                                                         clear_q ? 1 : 0);
}

void chem_launch_half4d(const ChemDev& D, const double* pos4, bool first, bool clear_q,
                        cudaStream_t st) {
    const int tb = 256;
    chem_half<double><<<(D.N + tb - 1) / tb, tb, 0, st>>>(D, pos4, 4, first ? 0.0 : 0.5 * D.dt,
                                                          clear_q ? 1 : 0);
}

void chem_launch_flux_d(const ChemDev& D, const int* cnt, const int* idx, const double* dist,
                        const double* dwdr, int kstride, const double* mass, const double* rho,
                        double t, cudaStream_t st) {
    const int tb = 128;
    chem_flux<double><<<(D.N + tb - 1) / tb, tb, 0, st>>>(D, cnt, idx, dist, dwdr, kstride,
                                                          mass, rho, t);
}

void chem_launch_flux_f(const ChemDev& D, const int* cnt, const int* idx, const float* dist,
                        const float* dwdr, int kstride, const float* mass, const float* rho,
                        double t, cudaStream_t st) {
    const int tb = 128;
    chem_flux<float><<<(D.N + tb - 1) / tb, tb, 0, st>>>(D, cnt, idx, dist, dwdr, kstride, mass,
                                                         rho, t);
}

}  // namespace spg
