// nsm.cu — NSM exact stochastic reaction-diffusion event loop on the GPU.
//
// Restates nsm_core__take_step (spatialpy/solvers/c_base/ssa_sdpd-c-
// simulation-engine/src/simulate_rdme.cpp:211-472) with the NRM queue
// contract of NRMConstant_v5 (src/NRMConstant_v5.cpp:27-281): every voxel
// holds its next-event time, an event redraws the times of the voxels it
// touches, events run in increasing (time, voxel) order.
//
// One warp owns one trajectory.  Per trajectory (HBM, or shared memory when
// the whole state fits): counts x[N][S] int32 voxel-major, leaf times
// [N padded to 32] as double bit patterns, and a 32-ary tournament tree of
// (time, voxel) nodes whose levels >= 1 always live in shared memory while the
// warp runs.  An event reads, in one round, the source voxel's counts,
// Ddiag, neighbour row, all species' cumulative weight rows and its leaf
// group; after the destination is chosen, a second round reads the
// destination's counts and leaf group.  The tree is then repaired from those
// registers and shared memory alone.
//
// Numerics: propensities, the selection scans and the exponential waiting
// times are single precision; event times (the clock) are double and are
// compared as 64-bit integers.  Philox blocks and waiting-time variates are
// produced 32 events at a time, one event per lane.  Compiled with
// -fmad=false, the arithmetic rounds exactly like the CPU oracle, so a GPU
// trajectory equals the oracle's event for event.
#include <cstdint>
#include <climits>

#include "common.cuh"
#include "nsm_prog.cuh"
#include "nsm_small.cuh"

namespace spg {

// mass-action propensity (reaction.py:260-313) in float: the generated
// C++'s operator order with the second-order division by vol replaced by a
// product with 1/vol: k*vol, k*A, (k*A*B)*(1/vol), (k*A*(A-1))*(1/vol)
__device__ __forceinline__ float prop(const NsmInstance& I, int r, int xa, int xb, float vol,
                                      float ivol, int type) {
    if (I.allowed && !I.allowed[r * (I.T + 1) + type]) return 0.0f;
    const float k = I.rate[r];
    switch (I.kind[r]) {
        case SP_RXN_ZERO: return k * vol;
        case SP_RXN_FIRST: return k * (float)xa;
        case SP_RXN_SECOND: return k * (float)xa * (float)xb * ivol;
        default: return k * (float)xa * (float)(xa - 1) * ivol;
    }
}

// Propensity of reaction r at voxel v, every lane of the warp alike: lane s
// holds x[s].  Custom propensity programs are evaluated at time t (the
// event's time; 0 at queue builds, as initialize_rxn_propensities passes,
// simulate_rdme.cpp:123-124) with the voxel's volume and data functions.
__device__ __forceinline__ float prop_w(const NsmInstance& I, int r, int xreg, float vol,
                                        float ivol, int type, int v, double t) {
    if (I.kind[r] == SP_RXN_CUSTOM) {
        if (I.allowed && !I.allowed[r * (I.T + 1) + type]) return 0.0f;
        auto xs = [&](int s) { return __shfl_sync(SP_FULL, xreg, s); };
        return (float)run_program(I.code + I.code_off[r], I.consts, I.data, I.N, v, xs,
                                  (double)vol, t, type);
    }
    const int ra = I.reac[2 * r], rb = I.reac[2 * r + 1];
    const int xa = __shfl_sync(SP_FULL, xreg, ra < 0 ? 0 : ra);
    const int xb = __shfl_sync(SP_FULL, xreg, rb < 0 ? 0 : rb);
    return prop(I, r, xa, xb, vol, ivol, type);
}

// Sums of a voxel's reaction propensities and diffusion rates in the engine's
// order (simulate_rdme.cpp:122-126, 142-150).  Lane s holds x[s] / Ddiag[s];
// every lane computes the same sums.
__device__ __forceinline__ void voxel_rates(const NsmInstance& I, int type, float vol, float ivol,
                                            int xreg, float ddreg, float& srr, float& sdr,
                                            int v, double t) {
    float a = 0.0f;
    for (int r = 0; r < I.R; r++) a = a + prop_w(I, r, xreg, vol, ivol, type, v, t);
    float d = 0.0f;
    for (int s = 0; s < I.S; s++) {
        const int xs = __shfl_sync(SP_FULL, xreg, s);
        const float ds = __shfl_sync(SP_FULL, ddreg, s);
        d = d + ds * (float)xs;
    }
    srr = a;
    sdr = d;
}

// ---------------------------------------------------------------------------
// queue build (NRMConstant_v5::build, :52-71): one thread per (traj, voxel)
// ---------------------------------------------------------------------------
__global__ void nsm_init_leaves(NsmTraj* trajs, const NsmInstance* insts, int ntraj,
                                double t0, uint32_t build_index) {
    const int j = blockIdx.y;
    if (j >= ntraj) return;
    NsmTraj& T = trajs[j];
    const NsmInstance& I = insts[T.inst];
    // the instance and trajectory fields the loop reads, held in registers
    // (the leaf stores below could otherwise alias them for the compiler)
    const int N = I.N, S = I.S, R = I.R, NT1 = I.level_off[1], stride = I.leaf_stride;
    const bool tree1 = I.levels >= 1, source = I.has_source != 0;
    const int* __restrict__ X = T.x;
    long long* __restrict__ leaf = T.leaf;
    long long* __restrict__ nt = T.node_t;
    int* __restrict__ ni = T.node_i;
    long long* __restrict__ n2 = T.node_t2;
    const uint32_t k0 = T.key0, k1 = T.key1;
    const float* __restrict__ ddiag = I.ddiag;
    const int lane = threadIdx.x & 31;
    // leaf_stride is a multiple of 32 and blocks hold whole warps, so every
    // lane of a warp runs the same iterations, over one voxel group
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < stride; v += gridDim.x * blockDim.x) {
        float a = 0.0f;
        long long tv = SP_INF_BITS;
        bool idle = false;
        if (v < N && !source) {
            // no molecules and no reaction that fires without reactants:
            // every propensity and diffusion rate is zero
            int any = 0;
            for (int s = 0; s < S; s++) any |= X[(size_t)v * S + s];
            idle = any == 0;
        }
        if (v < N && !idle) {
            float srr = 0.0f, sdr = 0.0f;
            const int* x = X + (size_t)v * S;
            const int type = I.type[v];
            for (int r = 0; r < R; r++) {
                if (I.kind[r] == SP_RXN_CUSTOM) {
                    if (I.allowed && !I.allowed[r * (I.T + 1) + type]) continue;
                    auto xs = [&](int s) { return x[s]; };
                    srr = srr + (float)run_program(I.code + I.code_off[r], I.consts, I.data, N, v,
                                                   xs, (double)I.vol[v], 0.0, type);
                    continue;
                }
                const int ra = I.reac[2 * r], rb = I.reac[2 * r + 1];
                srr = srr + prop(I, r, ra < 0 ? 0 : x[ra], rb < 0 ? 0 : x[rb], I.vol[v],
                                 I.ivol[v], type);
            }
            for (int s = 0; s < S; s++) sdr = sdr + ddiag[(size_t)v * S + s] * (float)x[s];
            a = srr + sdr;
            // a voxel without propensity gets an infinite time whatever its
            // draw, so its Philox block is skipped (sparse systems rebuild fast)
            if (a > 0.0f) {
                const u32x4 rr = philox4x32_10((uint32_t)v, build_index, 1u, 0u, k0, k1);
                tv = draw_time(t0, neglog_f(u32f(rr.x)), a);
            }
        }
        leaf[v] = tv;
        // the group's level-1 node (minimum) and second-smallest time, here
        // instead of a second pass over the leaves
        if (tree1) {
            long long t = tv;
            int i = v;
            warp_argmin(t, i);
            long long t2 = i == v ? SP_INF_BITS : tv;
            int i2 = i == v ? INT_MAX : v;
            warp_argmin(t2, i2);
            if (lane == 0) {
                nt[NT1 + (v >> 5)] = t;
                ni[NT1 + (v >> 5)] = i;
                n2[v >> 5] = t2;
            }
        }
        // running total (steers speculation only): the warp's 32 rates summed
        // in fp32, then one fp64 atomic per warp (the fp64 pipe is the
        // scarce one on this part)
        float af = a > 0.0f ? a : 0.0f;
        for (int o = 16; o > 0; o >>= 1) af += __shfl_xor_sync(SP_FULL, af, o);
        if (lane == 0 && af > 0.0f) atomicAdd(&T.a_tot, (double)af);
    }
}

// The same rebuild with the network unpacked once per block into shared
// memory (SmallNet<MS, MR>, the event kernels' variants; a block serves one
// trajectory): the rates come from rates_small, which sums the same terms
// in the same order as prop() above, so the leaves are the same bits.  Used
// for the per-step rebuild of a moving domain.
template <int MS, int MR, bool EX>
__global__ void __launch_bounds__(256) nsm_init_leaves_net(NsmTraj* trajs, const NsmInstance* insts,
                                                           int ntraj, double t0,
                                                           uint32_t build_index) {
    const int j = blockIdx.y;
    if (j >= ntraj) return;
    NsmTraj& T = trajs[j];
    const NsmInstance& I = insts[T.inst];
    __shared__ SmallNet<MS, MR> Q;
    if (threadIdx.x == 0) {
        Q.S = I.S;
        Q.R = I.R;
    }
    if (threadIdx.x < MR) {
        const int r = threadIdx.x;
        const bool on = EX || r < I.R;
        Q.kind[r] = on ? I.kind[r] : 0;
        Q.ra[r] = on ? I.reac[2 * r] : 0;
        Q.rb[r] = on ? I.reac[2 * r + 1] : 0;
        Q.rate[r] = on ? I.rate[r] : 0.0f;
        unsigned long long m = 0;
        if (on)
            for (int t = 0; t <= I.T && t < 64; t++)
                if (!I.allowed || I.allowed[r * (I.T + 1) + t]) m |= 1ull << t;
        Q.allowed[r] = m;
    }
    __syncthreads();
    const int N = I.N, S = I.S, NT1 = I.level_off[1], stride = I.leaf_stride;
    const bool tree1 = I.levels >= 1, source = I.has_source != 0;
    const int* __restrict__ X = T.x;
    long long* __restrict__ leaf = T.leaf;
    long long* __restrict__ nt = T.node_t;
    int* __restrict__ ni = T.node_i;
    long long* __restrict__ n2 = T.node_t2;
    const uint32_t k0 = T.key0, k1 = T.key1;
    const float* __restrict__ ddiag = I.ddiag;
    const int* __restrict__ vtype = I.type;
    const float* __restrict__ vvol = I.vol;
    const float* __restrict__ vivol = I.ivol;
    const int lane = threadIdx.x & 31;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < stride; v += gridDim.x * blockDim.x) {
        float a = 0.0f;
        long long tv = SP_INF_BITS;
        if (v < N) {
            int x[MS];
            float dd[MS];
            int any = 0;
#pragma unroll
            for (int s = 0; s < MS; s++) {
                const bool on = EX || s < S;
                x[s] = on ? X[(size_t)v * S + s] : 0;
                dd[s] = on ? ddiag[(size_t)v * S + s] : 0.0f;
                any |= x[s];
            }
            if (source || any != 0) {
                float srr, sdr;
                rates_small<MS, MR, EX>(Q, x, dd, vvol[v], vivol[v], vtype[v], srr, sdr);
                a = srr + sdr;
                if (a > 0.0f) {
                    const u32x4 rr = philox4x32_10((uint32_t)v, build_index, 1u, 0u, k0, k1);
                    tv = draw_time(t0, neglog_f(u32f(rr.x)), a);
                }
            }
        }
        leaf[v] = tv;
        if (tree1) {
            long long t = tv;
            int i = v;
            warp_argmin(t, i);
            long long t2 = i == v ? SP_INF_BITS : tv;
            int i2 = i == v ? INT_MAX : v;
            warp_argmin(t2, i2);
            if (lane == 0) {
                nt[NT1 + (v >> 5)] = t;
                ni[NT1 + (v >> 5)] = i;
                n2[v >> 5] = t2;
            }
        }
        float af = a > 0.0f ? a : 0.0f;
        for (int o = 16; o > 0; o >>= 1) af += __shfl_xor_sync(SP_FULL, af, o);
        if (lane == 0 && af > 0.0f) atomicAdd(&T.a_tot, (double)af);
    }
}

// ---------------------------------------------------------------------------
// event loop
// ---------------------------------------------------------------------------

// Repair the tree after leaves a (and b when `two`) changed.  ga/gb: leaf
// group values (lane l holds leaf (a & ~31) + l, resp. b's group) with the new
// times already substituted.  NT/NI: the warp's shared-memory tree.
__device__ __forceinline__ void tree_repair(const NsmInstance& I, long long* NT, int* NI, int lane,
                                            int a, long long ta_grp, int b, long long tb_grp,
                                            bool two, long long& rt, int& ri) {
    int ca = a >> 5, cb = two ? (b >> 5) : ca;
    long long t1 = ta_grp, t2 = tb_grp;
    int i1 = (ca << 5) + lane, i2 = (cb << 5) + lane;
    bool wlive = two && cb != ca;    // b's path still separate and changing
    for (int l = 1;; l++) {
        // reduce the children of nodes ca (and cb) at level l-1
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const long long u1 = __shfl_xor_sync(SP_FULL, t1, o);
            const int j1 = __shfl_xor_sync(SP_FULL, i1, o);
            const long long u2 = __shfl_xor_sync(SP_FULL, t2, o);
            const int j2 = __shfl_xor_sync(SP_FULL, i2, o);
            if (kless(u1, j1, t1, i1)) { t1 = u1; i1 = j1; }
            if (kless(u2, j2, t2, i2)) { t2 = u2; i2 = j2; }
        }
        const int off = I.level_off[l];
        if (wlive) {
            // b's node unchanged: its ancestors only change through a's path
            const bool same = NT[off + cb] == t2 && NI[off + cb] == i2;
            __syncwarp();
            if (lane == 1 && !same) { NT[off + cb] = t2; NI[off + cb] = i2; }
            if (same) wlive = false;
        }
        if (lane == 0) { NT[off + ca] = t1; NI[off + ca] = i1; }
        __syncwarp();
        if (l == I.levels) break;
        // next level: children of the parents
        const int pa = ca >> 5, pb = cb >> 5;
        const int sz = I.level_size[l];
        const int c1 = (pa << 5) + lane;
        t1 = c1 < sz ? NT[off + c1] : SP_INF_BITS;
        i1 = c1 < sz ? NI[off + c1] : INT_MAX;
        if (wlive && pb != pa) {
            const int c2 = (pb << 5) + lane;
            t2 = c2 < sz ? NT[off + c2] : SP_INF_BITS;
            i2 = c2 < sz ? NI[off + c2] : INT_MAX;
        } else {
            wlive = false;
            t2 = SP_INF_BITS;
            i2 = INT_MAX;
        }
        ca = pa;
        cb = pb;
    }
    rt = t1;
    ri = i1;
}

// SMEM_STATE: counts and leaves of the trajectory are staged in shared memory
// too (small domains); otherwise they stay in HBM.
template <bool REF, bool SMEM_STATE>
__global__ void __launch_bounds__(128) nsm_advance_generic(NsmTraj* trajs, const NsmInstance* insts,
                                                   int ntraj, int step_end, double dt,
                                                   long long budget, long long max_ns, int* work,
                                                   int warp_smem_bytes, const int* tlist) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    unsigned char* wsm = smem + (size_t)(threadIdx.x >> 5) * warp_smem_bytes;
    for (;;) {
        int j = 0;
        if (lane == 0) j = atomicAdd(work, 1);
        j = __shfl_sync(SP_FULL, j, 0);
        if (j >= ntraj) return;
        NsmTraj& T = trajs[tlist ? tlist[j] : j];
        if (T.status != SP_TRAJ_OK || T.step >= step_end) continue;
        const NsmInstance& I = insts[T.inst];
        const int S = I.S, K = I.K, NN = I.num_nodes;
        // stage the tree (and the state) in shared memory
        long long* NT = (long long*)wsm;
        int* NI = (int*)(NT + NN);
        for (int e = lane; e < NN; e += 32) { NT[e] = T.node_t[e]; NI[e] = T.node_i[e]; }
        long long* LF = T.leaf;
        int32_t* X = T.x;
        if (SMEM_STATE) {
            long long* sl = (long long*)(((uintptr_t)(NI + NN) + 15) & ~(uintptr_t)15);
            int32_t* sx = (int32_t*)(sl + I.leaf_stride);
            for (int e = lane; e < I.leaf_stride; e += 32) sl[e] = T.leaf[e];
            for (int e = lane; e < I.N * S; e += 32) sx[e] = T.x[e];
            LF = sl;
            X = sx;
        }
        __syncwarp();
        const bool prefetch = K <= 32 && S <= 4;
        uint64_t evn = T.evn;
        long long nrx = T.nrx, ndf = T.ndf;
        int step = T.step;
        int status = SP_TRAJ_OK, errv = -1;
        double tlast = T.t_last;
        long long nev = 0;
        unsigned long long t_start;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_start));
        long long rt = NT[I.level_off[I.levels]];
        int ri = NI[I.level_off[I.levels]];
        Rng32 rb = rng_block(evn & ~31ull, lane, T.key0, T.key1);
        while (step < step_end && status == SP_TRAJ_OK) {
            const double t_end = dt * (double)step + dt;   // simulate_rdme.cpp:67, 215
            const long long t_end_bits = __double_as_longlong(t_end);
            bool step_done = false;
            for (;;) {
                const long long tb = rt;
                const int v = ri;
                if (tb == SP_INF_BITS) { step_done = true; break; }
                if (!REF && tb > t_end_bits) { step_done = true; break; }
                if (nev >= budget) { status = SP_TRAJ_BUDGET_EXHAUSTED; break; }
                if ((nev & 1023) == 1023) {
                    unsigned long long now;
                    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
                    if ((long long)(now - t_start) > max_ns) {
                        status = SP_TRAJ_BUDGET_EXHAUSTED;
                        break;
                    }
                }
                const double tt = __longlong_as_double(tb);
                const int src = (int)(evn & 31);
                const float ua = __shfl_sync(SP_FULL, rb.ua, src);
                const float ub = __shfl_sync(SP_FULL, rb.ub, src);
                const float e0 = __shfl_sync(SP_FULL, rb.e0, src);
                const float e1 = __shfl_sync(SP_FULL, rb.e1, src);
                evn++;
                nev++;
                if ((evn & 31) == 0) rb = rng_block(evn, lane, T.key0, T.key1);
                // load phase 1: everything that depends on v only
                int xv = lane < S ? X[(size_t)v * S + lane] : 0;
                const float ddv = lane < S ? I.ddiag[(size_t)v * S + lane] : 0.0f;
                const int typev = I.type[v];
                const float volv = I.vol[v], ivolv = I.ivol[v];
                const int cnt = I.nbr_cnt[v];
                int nb = -1;
                float cf0 = 0.f, cf1 = 0.f, cf2 = 0.f, cf3 = 0.f;
                if (prefetch && lane < cnt) {
                    nb = I.nbr_idx[(size_t)v * K + lane];
                    const float* cr = I.cdf + (size_t)v * S * K + lane;
                    cf0 = cr[0];
                    if (S > 1) cf1 = cr[K];
                    if (S > 2) cf2 = cr[2 * K];
                    if (S > 3) cf3 = cr[3 * K];
                }
                long long lgv = LF[(v & ~31) + lane];
                float srr, sdr;
                voxel_rates(I, typev, volv, ivolv, xv, ddv, srr, sdr, v, tt);
                const float tot = srr + sdr;
                tlast = tt;
                if (ua * tot <= srr) {                           // :255 reaction
                    const float target = REF ? ua * srr : ua * tot;
                    float cum = 0.0f;
                    int re = -1, last = -1;
                    for (int q = 0; q < I.R; q++) {
                        const float a = prop_w(I, q, xv, volv, ivolv, typev, v, tt);
                        cum = cum + a;
                        if (a > 0.0f) {
                            last = q;
                            if (target <= cum) { re = q; break; }
                        }
                    }
                    if (re < 0) re = last;
                    if (re < 0) { status = SP_TRAJ_SELECT_OVERFLOW; errv = v; break; }
                    for (int q = I.jcN[re]; q < I.jcN[re + 1]; q++)   // :285-296
                        if (lane == I.irN[q]) xv += I.prN[q];
                    if (__any_sync(SP_FULL, lane < S && xv < 0)) {
                        status = SP_TRAJ_NEG_COUNT; errv = v; break;
                    }
                    if (lane < S) X[(size_t)v * S + lane] = xv;
                    voxel_rates(I, typev, volv, ivolv, xv, ddv, srr, sdr, v, tt);
                    const long long tv = draw_time(tt, e0, srr + sdr);
                    if (lane == (v & 31)) lgv = tv;
                    if (lane == 0) LF[v] = tv;
                    tree_repair(I, NT, NI, lane, v, lgv, v, lgv, false, rt, ri);
                    nrx++;
                } else {                                          // diffusion
                    const float target = REF ? ua * sdr : ua * tot - srr;
                    float cum = 0.0f;
                    int sp = -1, last = -1;
                    for (int s = 0; s < S; s++) {                 // :319-321
                        const int xs = __shfl_sync(SP_FULL, xv, s);
                        const float ds = __shfl_sync(SP_FULL, ddv, s);
                        const float wgt = ds * (float)xs;
                        cum = cum + wgt;
                        if (wgt > 0.0f) {
                            last = s;
                            if (target <= cum) { sp = s; break; }
                        }
                    }
                    if (sp < 0) sp = last;
                    if (sp < 0) { status = SP_TRAJ_SELECT_OVERFLOW; errv = v; break; }
                    const float target2 = ub * __shfl_sync(SP_FULL, ddv, sp);   // :353-354
                    int k = -1, lastk = -1;
                    if (prefetch) {
                        const float c = sp == 0 ? cf0 : sp == 1 ? cf1 : sp == 2 ? cf2 : cf3;
                        float pc = __shfl_up_sync(SP_FULL, c, 1);
                        if (lane == 0) pc = 0.0f;
                        const bool pos = lane < cnt && c > pc;
                        const unsigned bp = __ballot_sync(SP_FULL, pos);
                        const unsigned bh = __ballot_sync(SP_FULL, pos && c > target2);
                        if (bh) k = __ffs(bh) - 1;
                        else if (bp) lastk = 31 - __clz(bp);
                    } else {
                        const float* crow = I.cdf + ((size_t)v * S + sp) * K;
                        float carry = 0.0f;
                        for (int base = 0; base < cnt; base += 32) {   // :359-367
                            const int kk = base + lane;
                            const float c = kk < cnt ? crow[kk] : -1.0f;
                            float pc = __shfl_up_sync(SP_FULL, c, 1);
                            if (lane == 0) pc = carry;
                            const bool pos = kk < cnt && c > pc;
                            const unsigned bp = __ballot_sync(SP_FULL, pos);
                            const unsigned bh = __ballot_sync(SP_FULL, pos && c > target2);
                            if (bh) { k = base + __ffs(bh) - 1; break; }
                            if (bp) lastk = base + 31 - __clz(bp);
                            carry = __shfl_sync(SP_FULL, c, 31);
                        }
                    }
                    if (k < 0) k = lastk;
                    if (k < 0) { status = SP_TRAJ_SELECT_OVERFLOW; errv = v; break; }
                    const int w = prefetch ? __shfl_sync(SP_FULL, nb, k & 31)
                                           : I.nbr_idx[(size_t)v * K + k];
                    // load phase 2: the destination
                    int xw = lane < S ? X[(size_t)w * S + lane] : 0;
                    const float ddw = lane < S ? I.ddiag[(size_t)w * S + lane] : 0.0f;
                    const int typew = I.type[w];
                    // the engine evaluates the destination's reactions with the
                    // source voxel's volume (simulate_rdme.cpp:431-433)
                    const float volw = REF ? volv : I.vol[w];
                    const float ivolw = REF ? ivolv : I.ivol[w];
                    const bool samegrp = (w >> 5) == (v >> 5);
                    long long lgw = samegrp ? lgv : LF[(w & ~31) + lane];
                    // :394-402; a moving particle can list its own start-of-step
                    // point, and a move onto itself leaves the count unchanged
                    if (lane == sp && w != v) { xv -= 1; xw += 1; }
                    if (lane == sp) {
                        X[(size_t)v * S + sp] = xv;
                        X[(size_t)w * S + sp] = xw;
                    }
                    voxel_rates(I, typev, volv, ivolv, xv, ddv, srr, sdr, v, tt);
                    const long long tv = draw_time(tt, e0, srr + sdr);
                    voxel_rates(I, typew, volw, ivolw, xw, ddw, srr, sdr, w, tt);
                    const long long tw = draw_time(tt, e1, srr + sdr);
                    if (lane == (v & 31)) lgv = tv;
                    if (samegrp) {
                        if (lane == (w & 31)) lgv = tw;
                        lgw = lgv;
                    } else if (lane == (w & 31)) {
                        lgw = tw;
                    }
                    if (lane == 0) LF[v] = tv;
                    if (lane == 1) LF[w] = tw;
                    tree_repair(I, NT, NI, lane, v, lgv, w, lgw, true, rt, ri);
                    ndf++;
                }
                if (REF && tb > t_end_bits) { step_done = true; break; }   // :233
            }
            if (step_done) step++;
            else break;
        }
        __syncwarp();
        for (int e = lane; e < NN; e += 32) { T.node_t[e] = NT[e]; T.node_i[e] = NI[e]; }
        if (SMEM_STATE) {
            for (int e = lane; e < I.leaf_stride; e += 32) T.leaf[e] = LF[e];
            for (int e = lane; e < I.N * S; e += 32) T.x[e] = X[e];
        }
        if (lane == 0) {
            T.evn = evn;
            T.nrx = nrx;
            T.ndf = ndf;
            T.step = step;
            T.status = status;
            T.t_last = tlast;
            if (errv >= 0) T.err_voxel = errv;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Fast path for small networks (S <= MS, R <= MR): the voxel's counts and
// Ddiag are read as warp-uniform broadcasts into registers, the reaction
// table lives in registers, and the tree is repaired with 32-bit warp min
// reductions on (time high word, time low word, index).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void tree_repair_redux(const NsmInstance& I, long long* NT, int* NI,
                                                  int lane, int a, long long ta_grp, int b,
                                                  long long tb_grp, bool two, long long& rt,
                                                  int& ri) {
    int ca = a >> 5, cb = two ? (b >> 5) : ca;
    long long t1 = ta_grp, t2 = tb_grp;
    int i1 = (ca << 5) + lane, i2 = (cb << 5) + lane;
    bool wlive = two && cb != ca;
    for (int l = 1;; l++) {
        long long m1, m2 = SP_INF_BITS;
        int j1, j2 = INT_MAX;
        argmin_redux(t1, i1, m1, j1);
        if (wlive) argmin_redux(t2, i2, m2, j2);
        const int off = I.level_off[l];
        if (wlive) {
            const bool same = NT[off + cb] == m2 && NI[off + cb] == j2;
            __syncwarp();
            if (lane == 1 && !same) { NT[off + cb] = m2; NI[off + cb] = j2; }
            if (same) wlive = false;
        }
        if (lane == 0) { NT[off + ca] = m1; NI[off + ca] = j1; }
        __syncwarp();
        if (l == I.levels) { rt = m1; ri = j1; return; }
        const int pa = ca >> 5, pb = cb >> 5;
        const int sz = I.level_size[l];
        const int c1 = (pa << 5) + lane;
        t1 = c1 < sz ? NT[off + c1] : SP_INF_BITS;
        i1 = c1 < sz ? NI[off + c1] : INT_MAX;
        if (wlive && pb != pa) {
            const int c2 = (pb << 5) + lane;
            t2 = c2 < sz ? NT[off + c2] : SP_INF_BITS;
            i2 = c2 < sz ? NI[off + c2] : INT_MAX;
        } else {
            wlive = false;
        }
        ca = pa;
        cb = pb;
    }
}

template <bool REF, bool SMEM_STATE, int MS, int MR, bool EX>
__global__ void __launch_bounds__(128) nsm_advance_small(NsmTraj* trajs, const NsmInstance* insts,
                                                         int ntraj, int step_end, double dt,
                                                         long long budget, long long max_ns,
                                                         int* work, int warp_smem_bytes,
                                                         const int* tlist) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    unsigned char* wsm = smem + (size_t)(threadIdx.x >> 5) * warp_smem_bytes;
    for (;;) {
        int j = 0;
        if (lane == 0) j = atomicAdd(work, 1);
        j = __shfl_sync(SP_FULL, j, 0);
        if (j >= ntraj) return;
        NsmTraj& T = trajs[tlist ? tlist[j] : j];
        if (T.status != SP_TRAJ_OK || T.step >= step_end) continue;
        const NsmInstance& I = insts[T.inst];
        const int S = I.S, K = I.K, NN = I.num_nodes;
        SmallNet<MS, MR> Q;
        Q.S = S;
        Q.R = I.R;
#pragma unroll
        for (int r = 0; r < MR; r++) {
            const bool on = EX || r < I.R;
            Q.kind[r] = on ? I.kind[r] : 0;
            Q.ra[r] = on ? I.reac[2 * r] : 0;
            Q.rb[r] = on ? I.reac[2 * r + 1] : 0;
            Q.rate[r] = on ? I.rate[r] : 0.0f;
            unsigned long long m = 0;
            if (on) {
                for (int t = 0; t <= I.T && t < 64; t++)
                    if (!I.allowed || I.allowed[r * (I.T + 1) + t]) m |= 1ull << t;
            }
            Q.allowed[r] = m;
        }
        long long* NT = (long long*)wsm;
        int* NI = (int*)(NT + NN);
        for (int e = lane; e < NN; e += 32) { NT[e] = T.node_t[e]; NI[e] = T.node_i[e]; }
        long long* LF = T.leaf;
        int32_t* X = T.x;
        if (SMEM_STATE) {
            long long* sl = (long long*)(((uintptr_t)(NI + NN) + 15) & ~(uintptr_t)15);
            int32_t* sx = (int32_t*)(sl + I.leaf_stride);
            for (int e = lane; e < I.leaf_stride; e += 32) sl[e] = T.leaf[e];
            for (int e = lane; e < I.N * S; e += 32) sx[e] = T.x[e];
            LF = sl;
            X = sx;
        }
        __syncwarp();
        const bool prefetch = K <= 32;
        uint64_t evn = T.evn;
        long long nrx = T.nrx, ndf = T.ndf;
        int step = T.step;
        int status = SP_TRAJ_OK, errv = -1;
        double tlast = T.t_last;
        long long nev = 0;
        unsigned long long t_start;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_start));
        long long rt = NT[I.level_off[I.levels]];
        int ri = NI[I.level_off[I.levels]];
        Rng32 rbk = rng_block(evn & ~31ull, lane, T.key0, T.key1);
        while (step < step_end && status == SP_TRAJ_OK) {
            const double t_end = dt * (double)step + dt;   // simulate_rdme.cpp:67, 215
            const long long t_end_bits = __double_as_longlong(t_end);
            bool step_done = false;
            for (;;) {
                const long long tb = rt;
                const int v = ri;
                if (tb == SP_INF_BITS) { step_done = true; break; }
                if (!REF && tb > t_end_bits) { step_done = true; break; }
                if (nev >= budget) { status = SP_TRAJ_BUDGET_EXHAUSTED; break; }
                if ((nev & 1023) == 1023) {
                    unsigned long long now;
                    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
                    if ((long long)(now - t_start) > max_ns) {
                        status = SP_TRAJ_BUDGET_EXHAUSTED;
                        break;
                    }
                }
                const double tt = __longlong_as_double(tb);
                const int src = (int)(evn & 31);
                const float ua = __shfl_sync(SP_FULL, rbk.ua, src);
                const float ub = __shfl_sync(SP_FULL, rbk.ub, src);
                const float e0 = __shfl_sync(SP_FULL, rbk.e0, src);
                const float e1 = __shfl_sync(SP_FULL, rbk.e1, src);
                evn++;
                nev++;
                if ((evn & 31) == 0) rbk = rng_block(evn, lane, T.key0, T.key1);
                // load phase 1: uniform loads of the source voxel + its rows
                int xv[MS];
                float ddv[MS];
#pragma unroll
                for (int s = 0; s < MS; s++) {
                    xv[s] = (EX || s < S) ? X[(size_t)v * S + s] : 0;
                    ddv[s] = (EX || s < S) ? I.ddiag[(size_t)v * S + s] : 0.0f;
                }
                const int typev = I.type[v];
                const float volv = I.vol[v], ivolv = I.ivol[v];
                const int cnt = I.nbr_cnt[v];
                int nb = -1;
                float cf[MS];
#pragma unroll
                for (int s = 0; s < MS; s++) cf[s] = 0.0f;
                if (prefetch && lane < cnt) {
                    nb = I.nbr_idx[(size_t)v * K + lane];
                    const float* cr = I.cdf + (size_t)v * S * K + lane;
#pragma unroll
                    for (int s = 0; s < MS; s++)
                        if (EX || s < S) cf[s] = cr[s * K];
                }
                long long lgv = LF[(v & ~31) + lane];
                float srr, sdr;
                rates_small<MS, MR, EX>(Q, xv, ddv, volv, ivolv, typev, srr, sdr);
                const float tot = srr + sdr;
                tlast = tt;
                if (ua * tot <= srr) {                           // :255 reaction
                    const float target = REF ? ua * srr : ua * tot;
                    float cum = 0.0f;
                    int re = -1, last = -1;
#pragma unroll
                    for (int q = 0; q < MR; q++) {
                        if ((EX || q < Q.R) && re < 0) {
                            const float a = prop_small<MS, MR, EX>(Q, q, xv, volv, ivolv, typev);
                            cum = cum + a;
                            if (a > 0.0f) {
                                last = q;
                                if (target <= cum) re = q;
                            }
                        }
                    }
                    if (re < 0) re = last;
                    if (re < 0) { status = SP_TRAJ_SELECT_OVERFLOW; errv = v; break; }
                    bool neg = false;
                    for (int q = I.jcN[re]; q < I.jcN[re + 1]; q++) {   // :285-296
                        const int sp = I.irN[q], d = I.prN[q];
#pragma unroll
                        for (int s = 0; s < MS; s++)
                            if (s == sp) { xv[s] += d; neg |= xv[s] < 0; }
                    }
                    if (neg) { status = SP_TRAJ_NEG_COUNT; errv = v; break; }
                    if (lane < S) {
#pragma unroll
                        for (int s = 0; s < MS; s++)
                            if (s == lane) X[(size_t)v * S + s] = xv[s];
                    }
                    rates_small<MS, MR, EX>(Q, xv, ddv, volv, ivolv, typev, srr, sdr);
                    const long long tv = draw_time(tt, e0, srr + sdr);
                    if (lane == (v & 31)) lgv = tv;
                    if (lane == 0) LF[v] = tv;
                    tree_repair_redux(I, NT, NI, lane, v, lgv, v, lgv, false, rt, ri);
                    nrx++;
                } else {                                          // diffusion
                    const float target = REF ? ua * sdr : ua * tot - srr;
                    float cum = 0.0f;
                    int sp = -1, last = -1;
#pragma unroll
                    for (int s = 0; s < MS; s++) {                // :319-321
                        if ((EX || s < S) && sp < 0) {
                            const float wgt = ddv[s] * (float)xv[s];
                            cum = cum + wgt;
                            if (wgt > 0.0f) {
                                last = s;
                                if (target <= cum) sp = s;
                            }
                        }
                    }
                    if (sp < 0) sp = last;
                    if (sp < 0) { status = SP_TRAJ_SELECT_OVERFLOW; errv = v; break; }
                    const float target2 = ub * pickf<MS>(ddv, sp);   // :353-354
                    int k = -1, lastk = -1;
                    if (prefetch) {
                        const float c = pickf<MS>(cf, sp);
                        float pc = __shfl_up_sync(SP_FULL, c, 1);
                        if (lane == 0) pc = 0.0f;
                        const bool pos = lane < cnt && c > pc;
                        const unsigned bp = __ballot_sync(SP_FULL, pos);
                        const unsigned bh = __ballot_sync(SP_FULL, pos && c > target2);
                        if (bh) k = __ffs(bh) - 1;
                        else if (bp) lastk = 31 - __clz(bp);
                    } else {
                        const float* crow = I.cdf + ((size_t)v * S + sp) * K;
                        float carry = 0.0f;
                        for (int base = 0; base < cnt; base += 32) {   // :359-367
                            const int kk = base + lane;
                            const float c = kk < cnt ? crow[kk] : -1.0f;
                            float pc = __shfl_up_sync(SP_FULL, c, 1);
                            if (lane == 0) pc = carry;
                            const bool pos = kk < cnt && c > pc;
                            const unsigned bp = __ballot_sync(SP_FULL, pos);
                            const unsigned bh = __ballot_sync(SP_FULL, pos && c > target2);
                            if (bh) { k = base + __ffs(bh) - 1; break; }
                            if (bp) lastk = base + 31 - __clz(bp);
                            carry = __shfl_sync(SP_FULL, c, 31);
                        }
                    }
                    if (k < 0) k = lastk;
                    if (k < 0) { status = SP_TRAJ_SELECT_OVERFLOW; errv = v; break; }
                    const int w = prefetch ? __shfl_sync(SP_FULL, nb, k & 31)
                                           : I.nbr_idx[(size_t)v * K + k];
                    // load phase 2: the destination
                    int xw[MS];
                    float ddw[MS];
#pragma unroll
                    for (int s = 0; s < MS; s++) {
                        xw[s] = (EX || s < S) ? X[(size_t)w * S + s] : 0;
                        ddw[s] = (EX || s < S) ? I.ddiag[(size_t)w * S + s] : 0.0f;
                    }
                    const int typew = I.type[w];
                    // the engine evaluates the destination's reactions with the
                    // source voxel's volume (simulate_rdme.cpp:431-433)
                    const float volw = REF ? volv : I.vol[w];
                    const float ivolw = REF ? ivolv : I.ivol[w];
                    const bool samegrp = (w >> 5) == (v >> 5);
                    long long lgw = samegrp ? lgv : LF[(w & ~31) + lane];
                    int nxv = 0, nxw = 0;
#pragma unroll
                    for (int s = 0; s < MS; s++)                      // :394-402
                        if (s == sp) {
                            if (w != v) { xv[s] -= 1; xw[s] += 1; }   // a move onto itself
                            nxv = xv[s];
                            nxw = xw[s];
                        }
                    if (lane == 0) {
                        X[(size_t)v * S + sp] = nxv;
                        X[(size_t)w * S + sp] = nxw;
                    }
                    rates_small<MS, MR, EX>(Q, xv, ddv, volv, ivolv, typev, srr, sdr);
                    const long long tv = draw_time(tt, e0, srr + sdr);
                    rates_small<MS, MR, EX>(Q, xw, ddw, volw, ivolw, typew, srr, sdr);
                    const long long tw = draw_time(tt, e1, srr + sdr);
                    if (lane == (v & 31)) lgv = tv;
                    if (samegrp) {
                        if (lane == (w & 31)) lgv = tw;
                        lgw = lgv;
                    } else if (lane == (w & 31)) {
                        lgw = tw;
                    }
                    if (lane == 0) LF[v] = tv;
                    if (lane == 1) LF[w] = tw;
                    tree_repair_redux(I, NT, NI, lane, v, lgv, w, lgw, true, rt, ri);
                    ndf++;
                }
                if (REF && tb > t_end_bits) { step_done = true; break; }   // :233
            }
            if (step_done) step++;
            else break;
        }
        __syncwarp();
        for (int e = lane; e < NN; e += 32) { T.node_t[e] = NT[e]; T.node_i[e] = NI[e]; }
        if (SMEM_STATE) {
            for (int e = lane; e < I.leaf_stride; e += 32) T.leaf[e] = LF[e];
            for (int e = lane; e < I.N * S; e += 32) T.x[e] = X[e];
        }
        if (lane == 0) {
            T.evn = evn;
            T.nrx = nrx;
            T.ndf = ndf;
            T.step = step;
            T.status = status;
            T.t_last = tlast;
            if (errv >= 0) T.err_voxel = errv;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// outputs: one block per trajectory
// ---------------------------------------------------------------------------
__global__ void nsm_snapshot(const NsmTraj* trajs, const NsmInstance* insts, int ntraj,
                             int32_t* counts, const long long* count_off, long long* moments,
                             const long long* mom_off, int out_index) {
    const int j = blockIdx.x;
    if (j >= ntraj) return;
    const NsmTraj& T = trajs[j];
    const NsmInstance& I = insts[T.inst];
    const long long n = (long long)I.N * I.S;
    for (long long e = threadIdx.x; e < n; e += blockDim.x) {
        const int x = T.x[e];
        if (counts) counts[count_off[j] + (long long)out_index * n + e] = x;
        if (moments && x != 0) {
            long long* m = moments + 2 * (mom_off[T.inst] + (long long)out_index * n + e);
            atomicAdd((unsigned long long*)m, (unsigned long long)(long long)x);
            atomicAdd((unsigned long long*)(m + 1), (unsigned long long)((long long)x * x));
        }
    }
}

__global__ void nsm_copy_u0(NsmTraj* trajs, const NsmInstance* insts, int ntraj,
                            const uint32_t* const* u0) {
    const int j = blockIdx.y;
    if (j >= ntraj) return;
    NsmTraj& T = trajs[j];
    const NsmInstance& I = insts[T.inst];
    const long long n = (long long)I.N * I.S;
    const uint32_t* src = u0[T.inst];
    for (long long e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x)
        T.x[e] = (int32_t)src[e];
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
__global__ void nsm_reset_totals(NsmTraj* trajs, int ntraj) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < ntraj) trajs[j].a_tot = 0.0;
}

// levels 2..L of every trajectory's tree, one block per trajectory (these
// levels hold few nodes: a launch per level would cost more than the work)
__global__ void nsm_build_upper(NsmTraj* trajs, const NsmInstance* insts, int ntraj) {
    const int j = blockIdx.x;
    if (j >= ntraj) return;
    NsmTraj& T = trajs[j];
    const NsmInstance& I = insts[T.inst];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int l = 1; l < I.levels; l++) {
        const int nparent = I.level_size[l + 1];
        for (int p = wid; p < nparent; p += nw) {
            const int c = p * 32 + lane;
            long long t = SP_INF_BITS;
            int i = INT_MAX;
            if (c < I.level_size[l]) {
                t = T.node_t[I.level_off[l] + c];
                i = T.node_i[I.level_off[l] + c];
            }
            warp_argmin(t, i);
            if (lane == 0) {
                T.node_t[I.level_off[l + 1] + p] = t;
                T.node_i[I.level_off[l + 1] + p] = i;
            }
        }
        __syncthreads();
    }
}

// variant: the register-resident network of every trajectory (the event
// kernels' numbering: 1 <4, 8>, 2 <8, 16>, 3 exactly <1, 2>, 4 exactly <3, 4>),
// 0 for the generic rebuild
void launch_nsm_rebuild(NsmTraj* trajs, const NsmInstance* insts, int ntraj, int max_leaf,
                        int max_levels, double t0, uint32_t build_index, int variant,
                        cudaStream_t st) {
    const int gx = (max_leaf + 255) / 256 < 64 ? (max_leaf + 255) / 256 : 64;
    dim3 g(gx, ntraj);
    nsm_reset_totals<<<(ntraj + 127) / 128, 128, 0, st>>>(trajs, ntraj);
    switch (variant) {   // + level 1
        case 1: nsm_init_leaves_net<4, 8, false><<<g, 256, 0, st>>>(trajs, insts, ntraj, t0, build_index); break;
        case 2: nsm_init_leaves_net<8, 16, false><<<g, 256, 0, st>>>(trajs, insts, ntraj, t0, build_index); break;
        case 3: nsm_init_leaves_net<1, 2, true><<<g, 256, 0, st>>>(trajs, insts, ntraj, t0, build_index); break;
        case 4: nsm_init_leaves_net<3, 4, true><<<g, 256, 0, st>>>(trajs, insts, ntraj, t0, build_index); break;
        default: nsm_init_leaves<<<g, 256, 0, st>>>(trajs, insts, ntraj, t0, build_index); break;
    }
    if (max_levels > 1) nsm_build_upper<<<ntraj, 256, 0, st>>>(trajs, insts, ntraj);
}

// u0 copy, then (build_queue) the queue at t = 0 with build index 0; a
// moving domain builds its queues per step instead (launch_nsm_rebuild)
void launch_nsm_init(NsmTraj* trajs, const NsmInstance* insts, int ntraj, int max_leaf,
                     int max_levels, const uint32_t* const* u0, bool build_queue,
                     cudaStream_t st) {
    const int gx = (max_leaf + 255) / 256 < 64 ? (max_leaf + 255) / 256 : 64;
    dim3 g(gx, ntraj);
    if (u0) nsm_copy_u0<<<g, 256, 0, st>>>(trajs, insts, ntraj, u0);
    if (!build_queue) return;
    nsm_init_leaves<<<g, 256, 0, st>>>(trajs, insts, ntraj, 0.0, 0u);   // + level 1
    if (max_levels > 1) nsm_build_upper<<<ntraj, 256, 0, st>>>(trajs, insts, ntraj);
}

// Per-warp shared memory: the tree (12 bytes per node) and, for small
// domains, the leaves and counts.
int nsm_warp_smem(const NsmInstance& d, bool with_state) {
    size_t b = (size_t)d.num_nodes * 12;
    b = (b + 15) / 16 * 16;
    if (with_state) b += (size_t)d.leaf_stride * 8 + (size_t)d.N * d.S * 4;
    return (int)((b + 15) / 16 * 16);
}

typedef void (*AdvanceFn)(NsmTraj*, const NsmInstance*, int, int, double, long long, long long,
                          int*, int, const int*);

template <bool REF, bool SM>
static AdvanceFn pick_kernel(int variant) {
    switch (variant) {
        case 1: return nsm_advance_small<REF, SM, 4, 8, false>;
        case 2: return nsm_advance_small<REF, SM, 8, 16, false>;
        case 3: return nsm_advance_small<REF, SM, 1, 2, true>;
        case 4: return nsm_advance_small<REF, SM, 3, 4, true>;
        default: return nsm_advance_generic<REF, SM>;
    }
}

// variant: 0 generic (any S, R); 1 small (S <= 4, R <= 8); 2 small (S <= 8,
// R <= 16); 3 exactly S = 1, R = 2; 4 exactly S = 3, R = 4
// tlist: the trajectories to advance (ntraj entries, taken in order), or
// nullptr for 0..ntraj-1
void launch_nsm_advance(bool ref, bool smem_state, int variant, int warp_smem, int wpb,
                        NsmTraj* trajs, const NsmInstance* insts, int ntraj, int step_end,
                        double dt, long long budget, long long max_ns, int* work, int num_sms,
                        const int* tlist, cudaStream_t st) {
    cudaMemsetAsync(work, 0, sizeof(int), st);
    // one warp per block until every SM has a block
    if (ntraj <= 2 * num_sms) wpb = 1;
    int blocks = (ntraj + wpb - 1) / wpb;
    // persistent warps: enough resident blocks to cover the SMs several times
    const int per_sm = (200 * 1024) / (wpb * warp_smem) > 0 ? (200 * 1024) / (wpb * warp_smem) : 1;
    const int cap = num_sms * (per_sm < 16 ? per_sm : 16);
    if (blocks > cap) blocks = cap;
    const int smem = wpb * warp_smem;
    AdvanceFn fn = ref ? (smem_state ? pick_kernel<true, true>(variant) : pick_kernel<true, false>(variant))
                       : (smem_state ? pick_kernel<false, true>(variant) : pick_kernel<false, false>(variant));
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    fn<<<blocks, wpb * 32, smem, st>>>(trajs, insts, ntraj, step_end, dt, budget, max_ns, work,
                                       warp_smem, tlist);
}

void launch_nsm_snapshot(const NsmTraj* trajs, const NsmInstance* insts, int ntraj,
                         int32_t* counts, const long long* count_off, long long* moments,
                         const long long* mom_off, int out_index, cudaStream_t st) {
    nsm_snapshot<<<ntraj, 256, 0, st>>>(trajs, insts, ntraj, counts, count_off, moments, mom_off,
                                        out_index);
}

}  // namespace spg
