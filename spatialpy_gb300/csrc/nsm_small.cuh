// nsm_small.cuh — device helpers shared by the NSM event-loop kernels:
// waiting-time draws, per-lane Philox blocks, warp argmin by 32-bit
// reductions, and the register-resident small-network propensities.
#pragma once
#include <climits>

#include "common.cuh"

namespace spg {

// next firing time t + E/a (NRMConstant_v5.cpp:57, :98) as double bits
__device__ __forceinline__ long long draw_time(double t, float e, float a) {
    return a > 0.0f ? __double_as_longlong(t + (double)(e / a)) : SP_INF_BITS;
}

struct Rng32 {
    float ua, ub, e0, e1;   // this lane's event block values
};

__device__ __forceinline__ Rng32 rng_block(uint64_t base, int lane, uint32_t k0, uint32_t k1) {
    const uint64_t c = base + (uint64_t)lane;
    const u32x4 r = philox4x32_10((uint32_t)c, (uint32_t)(c >> 32), 0u, 0u, k0, k1);
    return Rng32{u24(r.x), u24(r.y), neglog_f(u32f(r.z)), neglog_f(u32f(r.w))};
}

__device__ __forceinline__ void argmin_redux(long long t, int i, long long& mt, int& mi) {
    const unsigned hi = (unsigned)((unsigned long long)t >> 32), lo = (unsigned)t;
    const unsigned mhi = __reduce_min_sync(SP_FULL, hi);
    const unsigned mlo = __reduce_min_sync(SP_FULL, hi == mhi ? lo : 0xffffffffu);
    const unsigned mid = __reduce_min_sync(SP_FULL, (hi == mhi && lo == mlo) ? (unsigned)i : 0xffffffffu);
    mt = (long long)(((unsigned long long)mhi << 32) | mlo);
    mi = (int)mid;
}

template <int MS>
__device__ __forceinline__ int pick(const int (&x)[MS], int s) {
    int r = x[0];
#pragma unroll
    for (int q = 1; q < MS; q++) r = s == q ? x[q] : r;
    return r;
}
template <int MS>
__device__ __forceinline__ float pickf(const float (&x)[MS], int s) {
    float r = x[0];
#pragma unroll
    for (int q = 1; q < MS; q++) r = s == q ? x[q] : r;
    return r;
}

template <int MS, int MR>
struct SmallNet {
    int S, R;
    int kind[MR], ra[MR], rb[MR];
    float rate[MR];
    unsigned long long allowed[MR];   // bit t: reaction may fire in type t (t < 64)
};

// EX: the network has exactly MS species and MR reactions (no guards).
// Branch-free mass action: ((k*A)*B)*W with A = vol (0th order) or x_a,
// B = x_b (2nd order), x_a - 1 (dimer) or 1, W = 1/vol (2nd order) or 1;
// the factors 1 are exact, so each kind rounds like its own expression.
template <int MS, int MR, bool EX>
__device__ __forceinline__ float prop_small(const SmallNet<MS, MR>& Q, int r, const int (&x)[MS],
                                            float vol, float ivol, int type) {
    const int kd = Q.kind[r];
    const int xa = pick<MS>(x, Q.ra[r]);
    const int xb = kd == SP_RXN_DIMER ? xa - 1 : pick<MS>(x, Q.rb[r]);
    const float A = kd == SP_RXN_ZERO ? vol : (float)xa;
    const float B = kd >= SP_RXN_SECOND ? (float)xb : 1.0f;
    const float W = kd >= SP_RXN_SECOND ? ivol : 1.0f;
    const float a = Q.rate[r] * A * B * W;
    return ((Q.allowed[r] >> type) & 1ull) ? a : 0.0f;
}

template <int MS, int MR, bool EX>
__device__ __forceinline__ void rates_small(const SmallNet<MS, MR>& Q, const int (&x)[MS],
                                            const float (&dd)[MS], float vol, float ivol, int type,
                                            float& srr, float& sdr) {
    float a = 0.0f;
#pragma unroll
    for (int r = 0; r < MR; r++)
        if (EX || r < Q.R) a = a + prop_small<MS, MR, EX>(Q, r, x, vol, ivol, type);
    float d = 0.0f;
#pragma unroll
    for (int s = 0; s < MS; s++)
        if (EX || s < Q.S) d = d + dd[s] * (float)x[s];
    srr = a;
    sdr = d;
}

}  // namespace spg
