// chem.cuh — deterministic chemistry interface (chem.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/spgpu.h"

namespace spg {

// device view of one instance's deterministic chemistry
struct ChemDev {
    int N, S, R, T;
    double dt, h;
    double* C;                 // [N][S]
    double* Q;                 // [N][S]
    const int* type;           // [N]
    const double* diffusion;   // [S][T] (solver.py:269-286)
    const int* stoich;         // [S][R] dense
    const uint8_t* allowed;    // [R][T+1] or nullptr
    const int32_t* code;       // ODE rate programs, SP_OP_X reads C
    const int32_t* code_off;   // [R+1]
    const double* consts;
    const double* data;        // [num_data][N]
    int nbc;
    const double* bc_box;      // [nbc][6]
    const int* bc_type;
    const int* bc_target;
    const double* bc_value;    // [nbc][3]
};

// first: no half step from the previous step's Q (step 0, simulate.cpp:81);
// pos: particle positions ([N][3] double, or 4-vectors of the flow)
void chem_launch_half(const ChemDev& D, const double* pos, bool first, bool clear_q,
                      cudaStream_t st);
void chem_launch_half4f(const ChemDev& D, const float* pos4, bool first, bool clear_q,
                        cudaStream_t st);
void chem_launch_half4d(const ChemDev& D, const double* pos4, bool first, bool clear_q,
                        cudaStream_t st);
void chem_launch_flux_d(const ChemDev& D, const int* cnt, const int* idx, const double* dist,
                        const double* dwdr, int kstride, const double* mass, const double* rho,
                        double t, cudaStream_t st);
void chem_launch_flux_f(const ChemDev& D, const int* cnt, const int* idx, const float* dist,
                        const float* dwdr, int kstride, const float* mass, const float* rho,
                        double t, cudaStream_t st);

}  // namespace spg
