// sdpd.cuh — SDPD particle-flow engine interface (sdpd.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "../../include/spgpu.h"

namespace spg {

struct SdpdState;

// Uploads the particle state of a moving-domain instance.  Returns nullptr
// (with *err set) on failure.
// self_step: a moved particle meets its own start-of-step point at |dt vt|
// (always so in FP32; in FP64 only when set, else from the rounded positions)
SdpdState* sdpd_create(const sp_scenario& s, int precision, int self_step, cudaStream_t st,
                       std::string* err);
void sdpd_destroy(SdpdState* s);
// nsteps engine steps (take_step substeps 0,1,2; simulate.cpp:33-48)
int sdpd_advance(SdpdState* s, int nsteps, double* ms, long long* launches, std::string* err);
int sdpd_get_state(SdpdState* s, double* x, double* v, double* rho, std::string* err);
int sdpd_copy_neighbors(SdpdState* s, int kmax, int* count, int* idx, double* dist, double* dwdr,
                        double* dij, std::string* err);

// Coupling with the NSM on a moving domain (simulate_threads.cpp:232-281):
// the lists of the last step's force pass with D_ij, and the flow state.
struct SdpdLists {
    int* count;      // [N]
    int* idx;        // [N][kcap]
    void* dij;       // [N][kcap] REAL (float, or double when f64)
    void* rho;       // [N] REAL
    void* dist;      // [N][kcap] REAL
    void* dwdr;      // [N][kcap] REAL
    void* mass;      // [N] REAL
    void* pos;       // [N] 4-vectors of REAL
    int kcap;
    bool f64;
    int step;        // steps taken
};
int sdpd_enable_dij(SdpdState* s, std::string* err);            // lists carry D_ij from now on
int sdpd_reset(SdpdState* s, std::string* err);                 // back to the initial state, step 0
void sdpd_enqueue_step(SdpdState* s);                           // one step, no host sync
constexpr int kSdpdLaunchesPerStep = 4;                       // kernels of one step
// one step in three parts: 0 predictor (take_step1), 1 lists + forces,
// 2 corrector (take_step2; advances the step counter); five kernels in all
void sdpd_enqueue_phase(SdpdState* s, int phase);
SdpdLists sdpd_lists(SdpdState* s);
// vol = m / rho, 1/vol = rho / m from the current densities (float)
void sdpd_launch_volumes(SdpdState* s, const double* mass, float* vol, float* ivol);
// device copies of the state in double (any pointer may be null)
void sdpd_launch_state_out(SdpdState* s, double* x, double* v, double* rho);
// synchronises; SP_OK or the error a step flagged (list overflow, NaN)
int sdpd_check_flag(SdpdState* s, std::string* err);

}  // namespace spg
