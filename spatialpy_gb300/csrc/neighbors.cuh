// neighbors.cuh — cell-list neighbour search interface (neighbors.cu).
#pragma once
#include <cuda_runtime.h>

namespace spg {

struct CellGrid {
    double lo[3];
    double cs;          // cell edge (>= h)
    int nc[3];
    int ncell;
    int dim;
};

CellGrid make_grid(const double* x_host, int n, int dim, double h);
int run_neighbor_search(const double* d_xq, const double* d_xt, int n, const CellGrid& g,
                        double h, const double* d_mass, const double* d_rho, int kmax,
                        int* d_count, int* d_idx, double* d_dist, double* d_dwdr, double* d_dij,
                        int* d_scratch_cell, int* d_hist, int* d_start, int* d_fill,
                        int* d_order, int* d_flag, cudaStream_t st);
void launch_diffusion_tables(int n, int S, int T, int kmax, const int* d_type, const int* d_count,
                             const int* d_idx, const double* d_dij, const double* d_diffusion,
                             float* d_ddiag, float* d_cdf, int2* d_cdfj, cudaStream_t st);
void launch_diffusion_tables_f32(int n, int S, int T, int kmax, const int* d_type,
                                 const int* d_count, const int* d_idx, const float* d_dij,
                                 const double* d_diffusion, float* d_ddiag, float* d_cdf,
                                 int2* d_cdfj, cudaStream_t st);

}  // namespace spg
