// neighbors.cu — fixed-radius neighbour search and SPH pair weights on the GPU.
//
// Replaces the ANN kd-tree search of Particle::find_neighbors
// (src/particle.cpp:240-294, external/ANN/src/kd_fix_rad_search.cpp:58-183)
// and the per-pair terms of Particle::add_to_neighbor_list
// (particle.cpp:150-210), then builds the diffusion tables of
// nsm_core__initialize_diff_propensities (simulate_rdme.cpp:131-152).
//
// Cell list: cells of edge >= h over the bounding box, built by a counting
// sort (key -> histogram -> exclusive scan -> scatter).  Each particle scans
// the 3^dim cells around it, keeps j when sum_d (q_d - p_d)^2 <= h^2 (summed in
// dimension order), the sum is non-zero (no self match) and sqrt(.) <= h, and
// stores the list sorted by (r^2, j).  Compiled with -fmad=false, so dist,
// dWdr and D_ij equal the reference engine's values bit for bit.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "common.cuh"
#include "neighbors.cuh"

namespace spg {

__device__ __forceinline__ int cell_coord(double p, const CellGrid& g, int d) {
    if (d >= g.dim) return 0;
    int c = (int)floor((p - g.lo[d]) / g.cs);
    c = c < 0 ? 0 : c;
    return c >= g.nc[d] ? g.nc[d] - 1 : c;
}

__global__ void cell_hist(const double* x, int n, CellGrid g, int* cell, int* hist) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int c = (cell_coord(x[3 * i], g, 0) * g.nc[1] + cell_coord(x[3 * i + 1], g, 1)) *
                          g.nc[2] + cell_coord(x[3 * i + 2], g, 2);
        cell[i] = c;
        atomicAdd(&hist[c], 1);
    }
}

// exclusive scan of hist[0..n) into start[0..n] by one block (set-up path)
__global__ void scan_single_block(const int* hist, int* start, int n) {
    __shared__ int warp_sums[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int base = 0; base < n; base += blockDim.x) {
        const int i = base + threadIdx.x;
        int v = i < n ? hist[i] : 0;
        int incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(SP_FULL, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) warp_sums[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            int ws = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(SP_FULL, ws, o);
                if (lane >= o) ws += t;
            }
            warp_sums[lane] = ws;
        }
        __syncthreads();
        const int before = (wid > 0 ? warp_sums[wid - 1] : 0) + carry;
        if (i < n) start[i] = before + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = before + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) start[n] = carry;
}

__global__ void cell_scatter(const int* cell, int n, const int* start, int* fill, int* order) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int c = cell[i];
        order[start[c] + atomicAdd(&fill[c], 1)] = i;
    }
}

// One thread per query particle.  xq: query points; xt: searched points.
template <int KCAP>
__global__ void neighbor_search_f64(const double* xq, const double* xt, int n, CellGrid g, double h,
                                    const double* mass, const double* rho, const int* start,
                                    const int* order, int kmax, int* count, int* idx, double* dist,
                                    double* dwdr, double* dij, int* overflow) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double cd2[KCAP];
    int cj[KCAP];
    const double q0 = xq[3 * i], q1 = xq[3 * i + 1], q2 = xq[3 * i + 2];
    const int c0 = cell_coord(q0, g, 0), c1 = cell_coord(q1, g, 1), c2 = cell_coord(q2, g, 2);
    const double sq = h * h;
    const int dim = g.dim;
    int m = 0;
    bool over = false;
    for (int a = c0 - 1; a <= c0 + 1; a++) {
        if (a < 0 || a >= g.nc[0]) continue;
        for (int b = c1 - 1; b <= c1 + 1; b++) {
            if (b < 0 || b >= g.nc[1]) continue;
            for (int c = c2 - 1; c <= c2 + 1; c++) {
                if (c < 0 || c >= g.nc[2]) continue;
                const int cid = (a * g.nc[1] + b) * g.nc[2] + c;
                for (int t = start[cid]; t < start[cid + 1]; t++) {
                    const int j = order[t];
                    // kd_fix_rad_search.cpp:160-170: sum (q-p)^2 in dimension order
                    double d2 = 0.0;
                    {
                        const double t0 = q0 - xt[3 * j];
                        d2 = d2 + t0 * t0;
                        if (dim > 1) {
                            const double t1 = q1 - xt[3 * j + 1];
                            d2 = d2 + t1 * t1;
                        }
                        if (dim > 2) {
                            const double t2 = q2 - xt[3 * j + 2];
                            d2 = d2 + t2 * t2;
                        }
                    }
                    if (d2 > sq || d2 == 0.0) continue;   // :173-174 no self match
                    if (sqrt(d2) > h) continue;           // particle.cpp:160-162
                    if (m >= KCAP || m >= kmax) { over = true; continue; }
                    int k = m++;
                    while (k > 0 && (d2 < cd2[k - 1] || (d2 == cd2[k - 1] && j < cj[k - 1]))) {
                        cd2[k] = cd2[k - 1];
                        cj[k] = cj[k - 1];
                        k--;
                    }
                    cd2[k] = d2;
                    cj[k] = j;
                }
            }
        }
    }
    if (over) atomicExch(overflow, 1);
    count[i] = m;
    // particle.cpp:165-187 (the engine's 1-D constant `5 / 4 * h` is h)
    const double alpha = dim == 3 ? 105 / (16 * M_PI * h * h * h)
                       : dim == 2 ? 5 / (M_PI * h * h) : 1 * h;
    for (int k = 0; k < m; k++) {
        const int j = cj[k];
        const double r2 = cd2[k];
        const double r = sqrt(r2);
        const double R = r / h;
        const double dW = alpha * (-12 * r / (h * h)) * ((1 - R) * (1 - R));
        const double ih = 1.0 / h;
        const double ihsq = ih * ih;
        const double dhr = h - r;
        const double wfd = -25.066903536973515383e0 * dhr * dhr * ihsq * ihsq * ihsq * ih;
        const double D = -2.0 * (mass[i] * mass[j]) / (mass[i] + mass[j]) * (rho[i] + rho[j]) /
                         (rho[i] * rho[j]) * r2 * wfd / (r2 + 0.01 * h * h);
        const size_t o = (size_t)i * kmax + k;
        idx[o] = j;
        if (dist) dist[o] = r;
        if (dwdr) dwdr[o] = dW;
        if (dij) dij[o] = D;
    }
}

// Ddiag[i,s] = sum_k D(s, type_j) D_ij (simulate_rdme.cpp:142-148) and the
// running sums over the list scanned by the destination choice (:359-367),
// accumulated in double in list order and rounded to float.  D_ij comes in
// double (static lists) or float (the FP32 flow's lists).
template <typename DT>
__global__ void diffusion_tables(int n, int S, int T, int kmax, const int* type, const int* count,
                                 const int* idx, const DT* dij, const double* diffusion,
                                 float* ddiag, float* cdf, int2* cdfj) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * S) return;
    const int i = e / S, s = e % S;
    double acc = 0.0;
    for (int k = 0; k < count[i]; k++) {
        const int j = idx[(size_t)i * kmax + k];
        const double dc = diffusion[s * T + (type[j] - 1)];
        acc = acc + dc * (double)dij[(size_t)i * kmax + k];
        const size_t o = ((size_t)i * S + s) * kmax + k;
        cdf[o] = (float)acc;
        cdfj[o] = make_int2(__float_as_int((float)acc), j);
    }
    ddiag[e] = (float)acc;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
CellGrid make_grid(const double* x_host, int n, int dim, double h) {
    CellGrid g{};
    g.dim = dim;
    g.cs = h * 1.0000001;
    double ext[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < 3; d++) {
        double lo = 0.0, hi = 0.0;
        if (d < dim && n > 0) {
            lo = hi = x_host[d];
            for (int i = 1; i < n; i++) {
                const double p = x_host[3 * i + d];
                lo = p < lo ? p : lo;
                hi = p > hi ? p : hi;
            }
        }
        g.lo[d] = std::isfinite(lo) ? lo : 0.0;
        ext[d] = d < dim && std::isfinite(hi - lo) ? hi - lo : 0.0;
    }
    // keep the grid modest: coarser cells only widen the candidate set.  The
    // counts are formed in double and bounded before the cast to int.
    auto cells = [&](double cs) {
        double c = 1.0;
        for (int d = 0; d < dim; d++) c *= std::floor(ext[d] / cs) + 1.0;
        return c;
    };
    if (!(g.cs > 0.0) || !std::isfinite(g.cs)) g.cs = 1.0;   // callers check h > 0
    while (!(cells(g.cs) <= (double)(1ll << 26))) g.cs *= 2.0;
    for (int d = 0; d < 3; d++) g.nc[d] = d < dim ? (int)(std::floor(ext[d] / g.cs) + 1.0) : 1;
    g.ncell = g.nc[0] * g.nc[1] * g.nc[2];
    return g;
}

// Full static search: returns 0, or 1 if some list exceeded kmax.
int run_neighbor_search(const double* d_xq, const double* d_xt, int n, const CellGrid& g,
                        double h, const double* d_mass, const double* d_rho, int kmax,
                        int* d_count, int* d_idx, double* d_dist, double* d_dwdr, double* d_dij,
                        int* d_scratch_cell, int* d_hist, int* d_start, int* d_fill,
                        int* d_order, int* d_flag, cudaStream_t st) {
    cudaMemsetAsync(d_hist, 0, sizeof(int) * g.ncell, st);
    cudaMemsetAsync(d_fill, 0, sizeof(int) * g.ncell, st);
    cudaMemsetAsync(d_flag, 0, sizeof(int), st);
    const int tb = 256, nb = (n + tb - 1) / tb;
    cell_hist<<<nb, tb, 0, st>>>(d_xt, n, g, d_scratch_cell, d_hist);
    scan_single_block<<<1, 1024, 0, st>>>(d_hist, d_start, g.ncell);
    cell_scatter<<<nb, tb, 0, st>>>(d_scratch_cell, n, d_start, d_fill, d_order);
    if (kmax <= 32)
        neighbor_search_f64<32><<<(n + 127) / 128, 128, 0, st>>>(
            d_xq, d_xt, n, g, h, d_mass, d_rho, d_start, d_order, kmax, d_count, d_idx, d_dist,
            d_dwdr, d_dij, d_flag);
    else if (kmax <= 64)
        neighbor_search_f64<64><<<(n + 127) / 128, 128, 0, st>>>(
            d_xq, d_xt, n, g, h, d_mass, d_rho, d_start, d_order, kmax, d_count, d_idx, d_dist,
            d_dwdr, d_dij, d_flag);
    else
        neighbor_search_f64<256><<<(n + 127) / 128, 128, 0, st>>>(
            d_xq, d_xt, n, g, h, d_mass, d_rho, d_start, d_order, kmax, d_count, d_idx, d_dist,
            d_dwdr, d_dij, d_flag);
    int flag = 0;
    cudaMemcpyAsync(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    return flag;
}

void launch_diffusion_tables(int n, int S, int T, int kmax, const int* d_type, const int* d_count,
                             const int* d_idx, const double* d_dij, const double* d_diffusion,
                             float* d_ddiag, float* d_cdf, int2* d_cdfj, cudaStream_t st) {
    const int e = n * S;
    diffusion_tables<double><<<(e + 255) / 256, 256, 0, st>>>(
        n, S, T, kmax, d_type, d_count, d_idx, d_dij, d_diffusion, d_ddiag, d_cdf, d_cdfj);
}

void launch_diffusion_tables_f32(int n, int S, int T, int kmax, const int* d_type,
                                 const int* d_count, const int* d_idx, const float* d_dij,
                                 const double* d_diffusion, float* d_ddiag, float* d_cdf,
                                 int2* d_cdfj, cudaStream_t st) {
    const int e = n * S;
    diffusion_tables<float><<<(e + 255) / 256, 256, 0, st>>>(
        n, S, T, kmax, d_type, d_count, d_idx, d_dij, d_diffusion, d_ddiag, d_cdf, d_cdfj);
}

}  // namespace spg

// ---------------------------------------------------------------------------
// Neighbour lists without device allocation.
//
// Some callers cannot allocate device memory while they run this path:
// code inside CUDA stream capture (cudaMalloc is not permitted there), and
// hosts that own a fixed device-memory arena and forbid allocation during a
// simulation step.  This entry point takes the caller's device buffers for
// inputs and outputs and keeps its own cell-list scratch in the file-scope
// array below, which every GPU that loads the library holds until the
// process exits.
// ---------------------------------------------------------------------------

namespace {
constexpr int kNoAllocMaxParticles = 262144;
constexpr int kNoAllocMaxCells = 524288;
// cell[P] | order[P] | hist[C] | fill[C] | start[C+1] | flag
constexpr size_t kNoAllocBytes =
    sizeof(int) * (2 * (size_t)kNoAllocMaxParticles + 3 * (size_t)kNoAllocMaxCells + 2);
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char sp_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {nullptr};

void noalloc_msg(char* err, int32_t errlen, const char* msg) {
    if (err && errlen > 0) {
        snprintf(err, (size_t)errlen, "%s", msg);
    }
}
}  // namespace

extern "C" int sp_neighbors_noalloc(const double* x, int32_t n, int32_t dim, double h,
                                    const double* mass, const double* rho, const double* lo,
                                    const double* hi, int32_t kmax, int32_t* count, int32_t* idx,
                                    double* dist, double* dWdr, double* Dij, void* stream,
                                    char* err, int32_t errlen) {
    using namespace spg;
    if (!x || !mass || !rho || !lo || !hi || !count || !idx || n < 1 || dim < 1 || dim > 3 ||
        !(h > 0.0) || !std::isfinite(h) || kmax < 1) {
        noalloc_msg(err, errlen, "sp_neighbors_noalloc: missing buffer or bad size");
        return SP_E_INVALID;
    }
    if (n > kNoAllocMaxParticles) {
        noalloc_msg(err, errlen, "sp_neighbors_noalloc: more than 262,144 particles");
        return SP_E_INVALID;
    }
    if (kmax > 256) {
        noalloc_msg(err, errlen, "sp_neighbors_noalloc: kmax above 256");
        return SP_E_INVALID;
    }
    CellGrid g{};
    g.dim = dim;
    g.cs = h * 1.0000001;
    // cell counts are formed in double and bounded before any cast to int
    double cells = 1.0;
    for (int d = 0; d < 3; d++) {
        g.lo[d] = d < dim ? lo[d] : 0.0;
        g.nc[d] = 1;
        if (d >= dim) continue;
        if (!std::isfinite(lo[d]) || !std::isfinite(hi[d])) {
            noalloc_msg(err, errlen, "sp_neighbors_noalloc: bounding box not finite");
            return SP_E_INVALID;
        }
        if (!(hi[d] >= lo[d])) {
            noalloc_msg(err, errlen, "sp_neighbors_noalloc: bounding box hi < lo");
            return SP_E_INVALID;
        }
        const double ext = std::floor((hi[d] - lo[d]) / g.cs) + 1.0;
        cells *= ext;
        if (!(ext <= (double)kNoAllocMaxCells) || !(cells <= (double)kNoAllocMaxCells)) {
            noalloc_msg(err, errlen,
                        "sp_neighbors_noalloc: more than 524,288 cells of edge h in the bounding box");
            return SP_E_INVALID;
        }
        g.nc[d] = (int)ext;
    }
    g.ncell = g.nc[0] * g.nc[1] * g.nc[2];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        noalloc_msg(err, errlen, "sp_neighbors_noalloc: no current CUDA device");
        return SP_E_CUDA;
    }
    void* base = nullptr;
    {
        // one-time set-up per device, with that device current
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            cudaError_t e = cudaGetSymbolAddress(&g_noalloc_ptr[dev], sp_noalloc_scratch);
            if (e != cudaSuccess) {
                g_noalloc_ptr[dev] = nullptr;
                noalloc_msg(err, errlen, "sp_neighbors_noalloc: cudaGetSymbolAddress failed");
                return SP_E_CUDA;
            }
        }
        base = g_noalloc_ptr[dev];
    }
    int* cell = (int*)base;
    int* order = cell + kNoAllocMaxParticles;
    int* hist = order + kNoAllocMaxParticles;
    int* fill = hist + kNoAllocMaxCells;
    int* start = fill + kNoAllocMaxCells;
    int* flag = start + kNoAllocMaxCells + 1;
    cudaStream_t st = (cudaStream_t)stream;
    // an error left on this thread by earlier, unrelated work is not this call's
    (void)cudaGetLastError();
    // the array keeps the previous call's contents: clear what starts at zero
    cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(int) * g.ncell, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(fill, 0, sizeof(int) * g.ncell, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(flag, 0, sizeof(int), st);
    if (e != cudaSuccess) {
        noalloc_msg(err, errlen, cudaGetErrorString(e));
        return SP_E_CUDA;
    }
    const int tb = 256, nb = (n + tb - 1) / tb;
    cell_hist<<<nb, tb, 0, st>>>(x, n, g, cell, hist);
    scan_single_block<<<1, 1024, 0, st>>>(hist, start, g.ncell);
    cell_scatter<<<nb, tb, 0, st>>>(cell, n, start, fill, order);
    const int sb = (n + 127) / 128;
    if (kmax <= 32)
        neighbor_search_f64<32><<<sb, 128, 0, st>>>(x, x, n, g, h, mass, rho, start, order, kmax,
                                                    count, idx, dist, dWdr, Dij, flag);
    else if (kmax <= 64)
        neighbor_search_f64<64><<<sb, 128, 0, st>>>(x, x, n, g, h, mass, rho, start, order, kmax,
                                                    count, idx, dist, dWdr, Dij, flag);
    else
        neighbor_search_f64<256><<<sb, 128, 0, st>>>(x, x, n, g, h, mass, rho, start, order, kmax,
                                                     count, idx, dist, dWdr, Dij, flag);
    int over = 0;
    e = cudaGetLastError();                                   // launch errors
    if (e == cudaSuccess) e = cudaMemcpyAsync(&over, flag, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        noalloc_msg(err, errlen, cudaGetErrorString(e));
        return SP_E_CUDA;
    }
    if (over) {
        noalloc_msg(err, errlen, "sp_neighbors_noalloc: a particle has more than kmax neighbours");
        return SP_E_UNSUPPORTED;
    }
    return SP_OK;
}
