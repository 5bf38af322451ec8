// nsm.cu — NSM exact stochastic reaction-diffusion event loop on the GPU.
//
// Restates nsm_core__take_step (spatialpy/solvers/c_base/ssa_sdpd-c-
// simulation-engine/src/simulate_rdme.cpp:211-472) with the NRM queue
// contract of NRMConstant_v5 (src/NRMConstant_v5.cpp:27-281): every voxel
// holds its next-event time, an event redraws the times of the voxels it
// touches, events run in increasing (time, voxel) order.
//
// Layout (per trajectory, HBM): counts x[N][S] int32 voxel-major; leaf
// times [N padded to 32] double; a 32-ary tournament tree of (time, voxel)
// nodes above the leaves.  One warp owns one trajectory; the 32 lanes load a
// voxel's species, a neighbour row or a tree group in one coalesced access
// and reduce with shuffles.
//
// Compiled with -fmad=false: the double-precision arithmetic (propensities,
// the selection scans, event times) rounds exactly like the CPU oracle, so a
// GPU trajectory equals the oracle's event for event.
#include <cstdint>
#include <climits>

#include "common.cuh"

namespace spg {

// mass-action propensity (reaction.py:260-313), operator order of the
// generated C++: k*vol, k*A, k*A*B/vol, k*A*(A-1)/vol
__device__ __forceinline__ double prop(const NsmInstance& I, int r, int xa, int xb, double vol,
                                       int type) {
    if (I.allowed && !I.allowed[r * (I.T + 1) + type]) return 0.0;
    const double k = I.rate[r];
    switch (I.kind[r]) {
        case SP_RXN_ZERO: return k * vol;
        case SP_RXN_FIRST: return k * (double)xa;
        case SP_RXN_SECOND: return k * (double)xa * (double)xb / vol;
        default: return k * (double)xa * (double)(xa - 1) / vol;
    }
}

// Sums of a voxel's reaction propensities and diffusion rates, in the
// engine's order (simulate_rdme.cpp:122-126, 142-150).  xreg / ddreg: lane s
// holds x[s] / Ddiag[s].  All lanes compute the same values.
__device__ __forceinline__ void voxel_rates(const NsmInstance& I, int type, double vol, int xreg,
                                            double ddreg, double& srr, double& sdr) {
    double a = 0.0;
    for (int r = 0; r < I.R; r++) {
        const int ra = I.reac[2 * r], rb = I.reac[2 * r + 1];
        const int xa = __shfl_sync(SP_FULL, xreg, ra < 0 ? 0 : ra);
        const int xb = __shfl_sync(SP_FULL, xreg, rb < 0 ? 0 : rb);
        a = a + prop(I, r, xa, xb, vol, type);
    }
    double d = 0.0;
    for (int s = 0; s < I.S; s++) {
        const int xs = __shfl_sync(SP_FULL, xreg, s);
        const double ds = __shfl_sync(SP_FULL, ddreg, s);
        d = d + ds * (double)xs;
    }
    srr = a;
    sdr = d;
}

__device__ __forceinline__ double draw_time(double t, double e, double a) {
    return a > 0.0 ? t + e / a : SP_INF;
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
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < I.leaf_stride;
         v += gridDim.x * blockDim.x) {
        if (v >= I.N) { T.leaf[v] = SP_INF; continue; }
        double srr = 0.0, sdr = 0.0;
        const int* x = T.x + (size_t)v * I.S;
        for (int r = 0; r < I.R; r++) {
            const int ra = I.reac[2 * r], rb = I.reac[2 * r + 1];
            srr = srr + prop(I, r, ra < 0 ? 0 : x[ra], rb < 0 ? 0 : x[rb], I.vol[v], I.type[v]);
        }
        for (int s = 0; s < I.S; s++) sdr = sdr + I.ddiag[(size_t)v * I.S + s] * (double)x[s];
        const u32x4 rr = philox4x32_10((uint32_t)v, build_index, 1u, 0u, T.key0, T.key1);
        T.leaf[v] = draw_time(t0, neglog(u01(rr.x)), srr + sdr);
    }
}

// one warp per parent node of level l+1
__global__ void nsm_build_level(NsmTraj* trajs, const NsmInstance* insts, int ntraj, int l) {
    const int j = blockIdx.y;
    if (j >= ntraj) return;
    NsmTraj& T = trajs[j];
    const NsmInstance& I = insts[T.inst];
    if (l >= I.levels) return;
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    const int nparent = I.level_size[l + 1];
    for (int p = blockIdx.x * wpb + (threadIdx.x >> 5); p < nparent; p += gridDim.x * wpb) {
        const int c = p * 32 + lane;
        double t = SP_INF;
        int i = INT_MAX;
        if (l == 0) {
            if (c < I.leaf_stride) { t = T.leaf[c]; i = c; }
        } else if (c < I.level_size[l]) {
            const TreeNode n = T.node[I.level_off[l] + c];
            t = n.t;
            i = n.i;
        }
        warp_argmin(t, i);
        if (lane == 0) T.node[I.level_off[l + 1] + p] = TreeNode{t, i, 0};
    }
}

// ---------------------------------------------------------------------------
// event loop: one warp per trajectory
// ---------------------------------------------------------------------------
struct WarpTree {
    double* leaf;
    TreeNode* node;
};

// Write the new times of voxels a (and b when `two`) and repair their paths
// to the root.  Returns the new root in (rt, ri).
__device__ __forceinline__ void tree_update(const NsmInstance& I, WarpTree W, int lane, int a,
                                            double ta, int b, double tb, bool two, double& rt,
                                            int& ri) {
    if (lane == 0) W.leaf[a] = ta;
    if (two && lane == 1) W.leaf[b] = tb;
    __syncwarp();
    int ca = a, cb = two ? b : a;
    double t1 = SP_INF, t2 = SP_INF;
    int i1 = INT_MAX, i2 = INT_MAX;
    for (int l = 0; l < I.levels; l++) {
        const int ga = ca >> 5, gb = cb >> 5;
        const int c1 = ga * 32 + lane, c2 = gb * 32 + lane;
        if (l == 0) {
            t1 = W.leaf[c1]; i1 = c1;
            t2 = W.leaf[c2]; i2 = c2;
        } else {
            const int sz = I.level_size[l];
            const TreeNode* L = W.node + I.level_off[l];
            if (c1 < sz) { const TreeNode n = L[c1]; t1 = n.t; i1 = n.i; } else { t1 = SP_INF; i1 = INT_MAX; }
            if (c2 < sz) { const TreeNode n = L[c2]; t2 = n.t; i2 = n.i; } else { t2 = SP_INF; i2 = INT_MAX; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double u1 = __shfl_xor_sync(SP_FULL, t1, o);
            const int j1 = __shfl_xor_sync(SP_FULL, i1, o);
            const double u2 = __shfl_xor_sync(SP_FULL, t2, o);
            const int j2 = __shfl_xor_sync(SP_FULL, i2, o);
            if (tless(u1, j1, t1, i1)) { t1 = u1; i1 = j1; }
            if (tless(u2, j2, t2, i2)) { t2 = u2; i2 = j2; }
        }
        TreeNode* P = W.node + I.level_off[l + 1];
        if (lane == 0) P[ga] = TreeNode{t1, i1, 0};
        if (lane == 1 && gb != ga) P[gb] = TreeNode{t2, i2, 0};
        __syncwarp();
        ca = ga;
        cb = gb;
    }
    rt = t1;
    ri = i1;
}

template <bool REF>
__global__ void __launch_bounds__(128) nsm_advance_seq(NsmTraj* trajs, const NsmInstance* insts,
                                                       int ntraj, int step_end, double dt,
                                                       long long budget, long long max_ns,
                                                       int* work) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        int j = 0;
        if (lane == 0) j = atomicAdd(work, 1);
        j = __shfl_sync(SP_FULL, j, 0);
        if (j >= ntraj) return;
        NsmTraj& T = trajs[j];
        if (T.status != SP_TRAJ_OK || T.step >= step_end) continue;
        const NsmInstance& I = insts[T.inst];
        const WarpTree W{T.leaf, T.node};
        int32_t* X = T.x;
        const int S = I.S, K = I.K;
        uint64_t evn = T.evn;
        long long nrx = T.nrx, ndf = T.ndf;
        int step = T.step;
        int status = SP_TRAJ_OK, errv = -1;
        double tlast = T.t_last;
        long long nev = 0;
        unsigned long long t_start;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_start));
        {
            const TreeNode rn = W.node[I.level_off[I.levels]];
            double rt = rn.t;
            int ri = rn.i;
            while (step < step_end && status == SP_TRAJ_OK) {
                const double t_end = dt * (double)step + dt;   // simulate_rdme.cpp:67, 215
                bool step_done = false;
                for (;;) {
                    const double tt = rt;
                    const int v = ri;
                    if (tt == SP_INF) { step_done = true; break; }
                    if (!REF && tt > t_end) { step_done = true; break; }
                    if (nev >= budget) { status = SP_TRAJ_BUDGET_EXHAUSTED; break; }
                    if ((nev & 1023) == 1023) {
                        unsigned long long now;
                        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
                        if ((long long)(now - t_start) > max_ns) {
                            status = SP_TRAJ_BUDGET_EXHAUSTED;
                            break;
                        }
                    }
                    const u32x4 rr = philox4x32_10((uint32_t)evn, (uint32_t)(evn >> 32), 0u, 0u,
                                                   T.key0, T.key1);
                    evn++;
                    nev++;
                    const double ua = u01(rr.x), ub = u01(rr.y);
                    const double e0 = neglog(u01(rr.z));
                    int xv = lane < S ? X[(size_t)v * S + lane] : 0;
                    const double ddv = lane < S ? I.ddiag[(size_t)v * S + lane] : 0.0;
                    const int typev = I.type[v];
                    const double volv = I.vol[v];
                    double srr, sdr;
                    voxel_rates(I, typev, volv, xv, ddv, srr, sdr);
                    const double tot = srr + sdr;
                    tlast = tt;
                    if (ua <= srr / tot) {                           // :255 reaction
                        const double target = REF ? ua * srr : ua * tot;
                        double cum = 0.0;
                        int re = -1, last = -1;
                        for (int q = 0; q < I.R; q++) {
                            const int ra = I.reac[2 * q], rb = I.reac[2 * q + 1];
                            const int xa = __shfl_sync(SP_FULL, xv, ra < 0 ? 0 : ra);
                            const int xb = __shfl_sync(SP_FULL, xv, rb < 0 ? 0 : rb);
                            const double a = prop(I, q, xa, xb, volv, typev);
                            cum = cum + a;
                            if (a > 0.0) {
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
                        voxel_rates(I, typev, volv, xv, ddv, srr, sdr);
                        const double tv = draw_time(tt, e0, srr + sdr);
                        tree_update(I, W, lane, v, tv, v, tv, false, rt, ri);
                        nrx++;
                    } else {                                          // diffusion
                        const double e1 = neglog(u01(rr.w));
                        const double target = REF ? ua * sdr : ua * tot - srr;
                        double cum = 0.0;
                        int sp = -1, last = -1;
                        for (int s = 0; s < S; s++) {                 // :319-321
                            const int xs = __shfl_sync(SP_FULL, xv, s);
                            const double ds = __shfl_sync(SP_FULL, ddv, s);
                            const double wgt = ds * (double)xs;
                            cum = cum + wgt;
                            if (wgt > 0.0) {
                                last = s;
                                if (target <= cum) { sp = s; break; }
                            }
                        }
                        if (sp < 0) sp = last;
                        if (sp < 0) { status = SP_TRAJ_SELECT_OVERFLOW; errv = v; break; }
                        const double target2 = ub * __shfl_sync(SP_FULL, ddv, sp);   // :353-354
                        const double* crow = I.cdf + ((size_t)v * S + sp) * K;
                        const int cnt = I.nbr_cnt[v];
                        int k = -1, lastk = -1;
                        double carry = 0.0;
                        for (int base = 0; base < cnt; base += 32) {  // :359-367
                            const int kk = base + lane;
                            const double c = kk < cnt ? crow[kk] : -1.0;
                            double pc = __shfl_up_sync(SP_FULL, c, 1);
                            if (lane == 0) pc = carry;
                            const bool pos = kk < cnt && c > pc;
                            const unsigned bp = __ballot_sync(SP_FULL, pos);
                            const unsigned bh = __ballot_sync(SP_FULL, pos && c > target2);
                            if (bh) { k = base + __ffs(bh) - 1; break; }
                            if (bp) lastk = base + 31 - __clz(bp);
                            carry = __shfl_sync(SP_FULL, c, 31);
                        }
                        if (k < 0) k = lastk;
                        if (k < 0) { status = SP_TRAJ_SELECT_OVERFLOW; errv = v; break; }
                        const int w = I.nbr_idx[(size_t)v * K + k];
                        int xw = lane < S ? X[(size_t)w * S + lane] : 0;
                        if (lane == sp) { xv -= 1; xw += 1; }               // :394-402
                        if (lane == sp) {
                            X[(size_t)v * S + sp] = xv;
                            X[(size_t)w * S + sp] = xw;
                        }
                        voxel_rates(I, typev, volv, xv, ddv, srr, sdr);
                        const double tv = draw_time(tt, e0, srr + sdr);
                        const double ddw = lane < S ? I.ddiag[(size_t)w * S + lane] : 0.0;
                        // the engine evaluates the destination's reactions with
                        // the source voxel's volume (simulate_rdme.cpp:431-433)
                        const double volw = REF ? volv : I.vol[w];
                        voxel_rates(I, I.type[w], volw, xw, ddw, srr, sdr);
                        const double tw = draw_time(tt, e1, srr + sdr);
                        tree_update(I, W, lane, v, tv, w, tw, true, rt, ri);
                        ndf++;
                    }
                    if (REF && tt > t_end) { step_done = true; break; }   // :233
                }
                if (step_done) step++;
                else break;
            }
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
        if (moments) {
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
void launch_nsm_init(NsmTraj* trajs, const NsmInstance* insts, int ntraj, int max_leaf,
                     int max_levels, const uint32_t* const* u0, cudaStream_t st) {
    dim3 g((max_leaf + 255) / 256 < 64 ? (max_leaf + 255) / 256 : 64, ntraj);
    if (u0) nsm_copy_u0<<<g, 256, 0, st>>>(trajs, insts, ntraj, u0);
    nsm_init_leaves<<<g, 256, 0, st>>>(trajs, insts, ntraj, 0.0, 0u);
    for (int l = 0; l < max_levels; l++) {
        dim3 gb((max_leaf / 32 + 3) / 4 + 1 < 64 ? (max_leaf / 32 + 3) / 4 + 1 : 64, ntraj);
        nsm_build_level<<<gb, 128, 0, st>>>(trajs, insts, ntraj, l);
    }
}

void launch_nsm_advance(bool ref, NsmTraj* trajs, const NsmInstance* insts, int ntraj,
                        int step_end, double dt, long long budget, long long max_ns, int* work,
                        int num_sms, cudaStream_t st) {
    cudaMemsetAsync(work, 0, sizeof(int), st);
    const int warps = ntraj;
    int blocks = (warps + 3) / 4;
    const int cap = num_sms * 16;
    if (blocks > cap) blocks = cap;
    if (ref)
        nsm_advance_seq<true><<<blocks, 128, 0, st>>>(trajs, insts, ntraj, step_end, dt, budget,
                                                      max_ns, work);
    else
        nsm_advance_seq<false><<<blocks, 128, 0, st>>>(trajs, insts, ntraj, step_end, dt, budget,
                                                       max_ns, work);
}

void launch_nsm_snapshot(const NsmTraj* trajs, const NsmInstance* insts, int ntraj,
                         int32_t* counts, const long long* count_off, long long* moments,
                         const long long* mom_off, int out_index, cudaStream_t st) {
    nsm_snapshot<<<ntraj, 256, 0, st>>>(trajs, insts, ntraj, counts, count_off, moments, mom_off,
                                        out_index);
}

}  // namespace spg
