// sdpd.cuh — SDPD particle-flow engine interface (sdpd.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "../../include/spgpu.h"

namespace spg {

struct SdpdState;

// Uploads the particle state of a moving-domain instance.  Returns nullptr
// (with *err set) on failure.
SdpdState* sdpd_create(const sp_scenario& s, int precision, cudaStream_t st, std::string* err);
void sdpd_destroy(SdpdState* s);
// nsteps engine steps (take_step substeps 0,1,2; simulate.cpp:33-48)
int sdpd_advance(SdpdState* s, int nsteps, double* ms, long long* launches, std::string* err);
int sdpd_get_state(SdpdState* s, double* x, double* v, double* rho, std::string* err);
int sdpd_copy_neighbors(SdpdState* s, int kmax, int* count, int* idx, double* dist, double* dwdr,
                        double* dij, std::string* err);

}  // namespace spg
