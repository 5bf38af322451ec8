// common.cuh — shared device helpers of libspgpu: Philox4x32-10 streams,
// the fixed-order -log(u), warp argmin, and the per-instance / per-trajectory
// device descriptors.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/spgpu.h"

#define SP_WARP 32
#define SP_FULL 0xffffffffu
#define SP_INF __longlong_as_double(0x7ff0000000000000ll)

namespace spg {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11).  Counter layout used by the engine:
//   events      : (event_index_lo, event_index_hi, 0, 0)
//   queue build : (voxel, build_index, 1, 0)
// key = (seed_lo, seed_hi).
// ---------------------------------------------------------------------------
struct u32x4 { uint32_t x, y, z, w; };

__host__ __device__ __forceinline__ u32x4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                                        uint32_t c3, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
#ifdef __CUDA_ARCH__
        const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
        const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
#else
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
        const uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return {c0, c1, c2, c3};
}

// u in (0,1): (r + 1/2) 2^-32, exact in double
__host__ __device__ __forceinline__ double u01(uint32_t r) {
    return ((double)r + 0.5) * (1.0 / 4294967296.0);
}

// -log(u) for u in (0,1): u = m 2^e, m in [sqrt(1/2), sqrt(2)), log m =
// 2 atanh((m-1)/(m+1)) by its Maclaurin series to w^10 (w = z^2), and
// e ln2 with ln2 split into a head whose low 21 mantissa bits are zero and a
// tail.  Every operation is an IEEE round-to-nearest op (the translation
// units using it are compiled without FMA contraction), so the result is
// bit-identical on every host and device that evaluates it in this order.
__host__ __device__ __forceinline__ double neglog(double u) {
#ifdef __CUDA_ARCH__
    long long b = __double_as_longlong(u);
#else
    long long b;
    __builtin_memcpy(&b, &u, 8);
#endif
    int e = (int)((b >> 52) & 0x7ff) - 1023;
    b = (b & 0x000fffffffffffffll) | 0x3ff0000000000000ll;
#ifdef __CUDA_ARCH__
    double m = __longlong_as_double(b);
#else
    double m;
    __builtin_memcpy(&m, &b, 8);
#endif
    if (m > 1.4142135623730951) { m = m * 0.5; e = e + 1; }
    const double z = (m - 1.0) / (m + 1.0);
    const double w = z * z;
    double p = 1.0 / 21.0;
    p = p * w + 1.0 / 19.0;
    p = p * w + 1.0 / 17.0;
    p = p * w + 1.0 / 15.0;
    p = p * w + 1.0 / 13.0;
    p = p * w + 1.0 / 11.0;
    p = p * w + 1.0 / 9.0;
    p = p * w + 1.0 / 7.0;
    p = p * w + 1.0 / 5.0;
    p = p * w + 1.0 / 3.0;
    p = p * w + 1.0;
    const double logm = (2.0 * z) * p;
    const double ln2_hi = 6.931471803691238e-01;
    const double ln2_lo = 1.9082149292705877e-10;
    const double ed = (double)e;
    return -(ed * ln2_hi + (ed * ln2_lo + logm));
}

// Selection uniform in (0,1) from the top 24 bits, exact in float.
__host__ __device__ __forceinline__ float u24(uint32_t r) {
    return (float)(r >> 8) * (1.0f / 16777216.0f) + (1.0f / 33554432.0f);
}
// Uniform in (0,1] for exponential draws, full 32-bit resolution near 0.
__host__ __device__ __forceinline__ float u32f(uint32_t r) {
    return ((float)r + 0.5f) * (1.0f / 4294967296.0f);
}

// Single-precision -log(u): the construction of neglog() in float (series to
// w^5, ln 2 head with 9 low mantissa bits cleared).  The NSM waiting times use
// it; the CPU oracle evaluates the same operations in the same order.
__host__ __device__ __forceinline__ float neglog_f(float u) {
#ifdef __CUDA_ARCH__
    unsigned b = __float_as_uint(u);
#else
    unsigned b;
    __builtin_memcpy(&b, &u, 4);
#endif
    int e = (int)((b >> 23) & 0xff) - 127;
    b = (b & 0x007fffffu) | 0x3f800000u;
#ifdef __CUDA_ARCH__
    float m = __uint_as_float(b);
#else
    float m;
    __builtin_memcpy(&m, &b, 4);
#endif
    if (m > 1.41421356f) { m = m * 0.5f; e = e + 1; }
    const float z = (m - 1.0f) / (m + 1.0f);
    const float w = z * z;
    float p = 1.0f / 11.0f;
    p = p * w + 1.0f / 9.0f;
    p = p * w + 1.0f / 7.0f;
    p = p * w + 1.0f / 5.0f;
    p = p * w + 1.0f / 3.0f;
    p = p * w + 1.0f;
    const float logm = (2.0f * z) * p;
    const float ed = (float)e;
    return -(ed * 0.693145751953125f + (ed * 1.428606765330187e-06f + logm));
}

// Event times are non-negative doubles or +inf; their IEEE bit patterns order
// like the values, so the queue compares them as 64-bit integers.
#define SP_INF_BITS 0x7ff0000000000000ll

// (time, index) lexicographic order of the event queue
__device__ __forceinline__ bool kless(long long ta, int ia, long long tb, int ib) {
    return ta < tb || (ta == tb && ia < ib);
}

__device__ __forceinline__ void warp_argmin(long long& t, int& i) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const long long t2 = __shfl_xor_sync(SP_FULL, t, o);
        const int i2 = __shfl_xor_sync(SP_FULL, i, o);
        if (kless(t2, i2, t, i)) { t = t2; i = i2; }
    }
}

constexpr int kMaxLevels = 8;

// Static (per model instance) device data of the NSM.
struct NsmInstance {
    int32_t N, S, R, T, K;            // voxels, species, reactions, types, neighbour stride
    int32_t levels;                   // tree levels above the leaves (root = level `levels`)
    int32_t level_size[kMaxLevels + 1];
    int32_t level_off[kMaxLevels + 1];  // node offset of level l (l >= 1) in the node arrays
    int32_t num_nodes;
    int32_t leaf_stride;              // padded leaf count (multiple of 32)
    const int32_t* type;              // [N]
    const float* vol;                 // [N] mass/rho rounded to float
    const float* ivol;                // [N] rho/mass rounded to float
    const int32_t* nbr_cnt;           // [N]
    const int32_t* nbr_idx;           // [N*K]
    const float* cdf;                 // [N*S*K] running sums of D(s,type_j) D_ij
    const int2* cdfj;                 // [N*S*K] (running sum as float bits, neighbour index)
    const float* ddiag;               // [N*S]
    const float* rate;                // [R] rate constants rounded to float
    const int32_t* kind;              // [R]
    const int32_t* reac;              // [2R]
    const uint8_t* allowed;           // [R*(T+1)] or nullptr
    const int32_t* jcN;               // [R+1]
    const int32_t* irN;
    const int32_t* prN;
    // custom propensities (SP_RXN_CUSTOM), or nullptr
    const int32_t* code;              // programs, concatenated
    const int32_t* code_off;          // [R+1]
    const double* consts;
    const double* data;               // [num_data * N] data function values
    int32_t num_data;
    int32_t has_custom;
    int32_t has_source;               // a zero-order or custom reaction: a voxel
                                      // without molecules may still have propensity
};

// Per-trajectory mutable state (device resident for the whole run).
struct NsmTraj {
    int32_t inst;
    int32_t status;                   // SP_TRAJ_*
    int32_t step;                     // next engine step to simulate
    int32_t err_voxel;
    uint32_t key0, key1;              // Philox key (seed)
    uint64_t evn;                     // event counter (Philox counter)
    int64_t nrx, ndf;                 // reaction / diffusion events
    double t_last;                    // time of the last executed event
    int32_t* x;                       // [N*S] counts
    long long* leaf;                  // [leaf_stride] next-event times (double bits)
    long long* node_t;                // [num_nodes] tree times, levels >= 1
    int32_t* node_i;                  // [num_nodes] tree voxel indices
    long long* node_t2;               // [level_size[1]] second-smallest leaf time per group
    double a_tot;                     // running sum of all voxel propensities (batch horizon)
    float bscale;                     // events aimed for per batch horizon (adapted)
    int32_t pad2;
    int64_t nbatch, ncand;            // speculative batches and their candidates
};

}  // namespace spg

#define SP_CUDA_TRY(expr)                                                  \
    do {                                                                    \
        cudaError_t _e = (expr);                                            \
        if (_e != cudaSuccess) {                                            \
            return ::spg_set_cuda_error(h, _e, #expr, __FILE__, __LINE__);  \
        }                                                                   \
    } while (0)
