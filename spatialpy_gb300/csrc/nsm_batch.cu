// nsm_batch.cu — speculative batched NSM event loop (one warp per trajectory).
//
// Same events, same order and same random numbers as the sequential event
// loop of nsm.cu (and the CPU oracle), executed up to 32 at a time:
//
//  1. candidates: the level-1 tree nodes (each the minimum of a group of 32
//     voxels) whose next-event time lies below a horizon theta, found
//     top-down through the shared-memory tree and sorted by (time, voxel).
//     theta = t_min + c / A, A the running FP64 sum of all voxel
//     propensities and c ~ 20 (adapted to the candidate counts seen).
//  2. each lane executes candidate i as the (n+i)-th event of the
//     trajectory: Philox counter n+i, reaction or diffusion choice, new
//     counts, and redrawn times for the voxels it touches.
//  3. the accepted prefix: candidate i is the sequential algorithm's next
//     event iff every earlier candidate j leaves all of its redrawn times and
//     the second-smallest time of its own voxel group above t_i, and no two
//     of the first i+1 events touch the same voxel.
//  4. the accepted events are written, the voxel groups they touched are
//     rescanned (minimum and second minimum), and the tree above them is
//     repaired.
//
// Rejected lanes leave no trace; their events are redone by a later batch
// with the same counters.  Compiled with -fmad=false (same rounding as the
// sequential kernel and the oracle).
#include <climits>
#include <cstdint>

#include "nsm_batch.cuh"

namespace spg {

// per-warp shared memory of the one-warp batch kernel
int nsm_batch_smem(const NsmInstance& d) { return nsm_batch_smem_w1(d); }

template <bool REF, int MS, int MR, bool EX>
__global__ void __launch_bounds__(32, 1) nsm_advance_batch(NsmTraj* trajs, const NsmInstance* insts,
                                                        int ntraj, int step_end, double dt,
                                                        long long budget, long long max_ns,
                                                        int* work, const int* tlist) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const unsigned ltm = (1u << lane) - 1u;
    for (;;) {
        int jt = 0;
        if (lane == 0) jt = atomicAdd(work, 1);
        jt = __shfl_sync(SP_FULL, jt, 0);
        if (jt >= ntraj) return;
        NsmTraj& T = trajs[tlist ? tlist[jt] : jt];
        if (T.status != SP_TRAJ_OK || T.step >= step_end) continue;
        const NsmInstance& I = insts[T.inst];
        const int S = I.S, K = I.K, NN = I.num_nodes, N1 = I.level_size[1], L = I.levels;
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
            if (on)
                for (int t = 0; t <= I.T && t < 64; t++)
                    if (!I.allowed || I.allowed[r * (I.T + 1) + t]) m |= 1ull << t;
            Q.allowed[r] = m;
        }
        long long* NT = (long long*)smem;
        long long* T2 = NT + NN;
        int* NI = (int*)(T2 + N1);
        int* fa = (int*)(NI + NN);
        int* fb = fa + kFront;
        int* flg = fb + kFront;     // repair flags of levels >= 2, all zero between batches
        const int flg_base = I.level_off[2];
        for (int e = lane; e < NN - I.level_size[1]; e += 32) flg[e] = 0;
        for (int e = lane; e < NN; e += 32) { NT[e] = T.node_t[e]; NI[e] = T.node_i[e]; }
        for (int e = lane; e < N1; e += 32) T2[e] = T.node_t2[e];
        __syncwarp();
        long long* LF = T.leaf;
        int32_t* X = T.x;
        uint64_t evn = T.evn;
        long long nrx = T.nrx, ndf = T.ndf;
        int step = T.step;
        int status = SP_TRAJ_OK, errv = -1;
        double tlast = T.t_last;
        double A = T.a_tot;
        float bsc = T.bscale;
        long long nev = 0;
        int nbatch = 0;
        long long stat_b = 0, stat_c = 0;
        unsigned long long t_start;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_start));
        long long rt = NT[I.level_off[L]];
        int ri = NI[I.level_off[L]];
        while (step < step_end && status == SP_TRAJ_OK) {
            const double t_end = dt * (double)step + dt;   // simulate_rdme.cpp:67, 215
            const long long t_end_bits = __double_as_longlong(t_end);
            bool step_done = false;
            for (;;) {
                if (rt == SP_INF_BITS) { step_done = true; break; }
                const bool over = rt > t_end_bits;
                if (over && !REF) { step_done = true; break; }
                if (nev >= budget) { status = SP_TRAJ_BUDGET_EXHAUSTED; break; }
                if ((++nbatch & 15) == 0) {
                    unsigned long long now;
                    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
                    if ((long long)(now - t_start) > max_ns) {
                        status = SP_TRAJ_BUDGET_EXHAUSTED;
                        break;
                    }
                }
                // ---- 1. candidates -------------------------------------------
                long long ct = SP_INF_BITS, ct2 = SP_INF_BITS;
                int ci = INT_MAX, count = 1;
                if (over) {   // the reference's one event past the step end, alone
                    if (lane == 0) { ct = rt; ci = ri; ct2 = T2[ri >> 5]; }
                } else {
                    float delta = A > 0.0 ? bsc / (float)A : 3.0e38f;
                    if (!(delta > 0.0f)) delta = 3.0e38f;
                    const double th = __longlong_as_double(rt) + (double)delta;
                    long long thb = __double_as_longlong(th);
                    if (thb > t_end_bits + 1) thb = t_end_bits + 1;   // no event past t_end
                    if (thb <= rt) thb = rt + 1;
                    count = batch_extract(I, NT, NI, fa, fb, lane, ltm, thb, ct, ci);
                    if (count < 0) {
                        if (bsc > 1.0f) { bsc *= 0.5f; continue; }
                        count = 1;        // degenerate: the minimum alone
                        ct = lane == 0 ? rt : SP_INF_BITS;
                        ci = lane == 0 ? ri : INT_MAX;
                    } else {
                        bitonic32(lane, ct, ci);
                    }
                    // the second-smallest time of each candidate's voxel group
                    ct2 = lane < count ? T2[ci >> 5] : SP_INF_BITS;
                    if (count >= 28) bsc = bsc * 0.8f;
                    else if (count < 16 && bsc < 64.0f) bsc = bsc * 1.25f;
                }
                stat_b++;
                stat_c += count;
                // ---- 2. speculative execution, one candidate per lane ----------
                const bool act = lane < count;
                Cand<MS> Cd;
                batch_execute<REF, MS, MR, EX>(I, Q, X, act, ci, ct, evn + (uint64_t)lane, T.key0,
                                               T.key1, Cd);
                const int v = Cd.v, w = Cd.w, sp = Cd.sp, err = Cd.err;
                const bool rxn = Cd.rxn;
                const long long tv = Cd.tv, tw = Cd.tw;
                const float dA = Cd.dA;
                int xv[MS], xw[MS];
#pragma unroll
                for (int s = 0; s < MS; s++) {
                    xv[s] = Cd.xv[s];
                    xw[s] = Cd.xw[s];
                }
                // ---- 3. the accepted prefix ------------------------------------
                long long bound = act ? ct2 : SP_INF_BITS;
                if (tv < bound) bound = tv;
                if (tw < bound) bound = tw;
                long long pm = bound;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const long long u = __shfl_up_sync(SP_FULL, pm, o);
                    if (lane >= o && u < pm) pm = u;
                }
                long long ex = __shfl_up_sync(SP_FULL, pm, 1);
                if (lane == 0) ex = SP_INF_BITS;
                bool conf = false;
                for (int q = 0; q < count; q++) {
                    const int vq = __shfl_sync(SP_FULL, v, q);
                    const int wq = __shfl_sync(SP_FULL, w, q);
                    if (q < lane) conf |= (v == wq) || (w >= 0 && (w == vq || w == wq));
                }
                const bool valid = act && ct < ex && !conf && (nev + lane) < budget;
                const unsigned vb = __ballot_sync(SP_FULL, valid);
                int m = vb == SP_FULL ? 32 : __ffs(~vb) - 1;
                const unsigned eb = __ballot_sync(SP_FULL, act && err != 0 && lane < m);
                if (eb) {
                    const int el = __ffs(eb) - 1;
                    status = __shfl_sync(SP_FULL, err, el);
                    errv = __shfl_sync(SP_FULL, v, el);
                    m = el;
                }
                // ---- 4. commit --------------------------------------------------
                const bool acc = lane < m;
                if (acc) {
#pragma unroll
                    for (int s = 0; s < MS; s++)
                        if (EX || s < S) X[(size_t)v * S + s] = xv[s];
                    LF[v] = tv;
                    if (w >= 0) {
#pragma unroll
                        for (int s = 0; s < MS; s++)
                            if (s == sp) X[(size_t)w * S + s] = xw[s];
                        LF[w] = tw;
                    }
                }
                nrx += __popc(__ballot_sync(SP_FULL, acc && rxn));
                ndf += __popc(__ballot_sync(SP_FULL, acc && !rxn));
                evn += (uint64_t)m;
                nev += m;
                if (m > 0) tlast = __longlong_as_double(__shfl_sync(SP_FULL, ct, m - 1));
                double dsum = acc ? (double)dA : 0.0;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) dsum += __shfl_xor_sync(SP_FULL, dsum, o);
                A += dsum;
                __syncwarp();
                // ---- 5. tree repair ---------------------------------------------
                // every accepted lane rescans its source group and, when it
                // differs, its destination group (32 contiguous leaves each)
                const int gv = v >> 5;
                const int gw = (w >= 0 && (w >> 5) != gv) ? w >> 5 : -1;
                if (acc) lane_rescan2(I, LF, NT, NI, T2, gv, gw);
                __syncwarp();
                // parents of changed nodes, level by level: one lane per
                // changed node on wide levels, the whole level by warp
                // reductions on levels of at most 8 nodes
                int pa = acc ? gv : -1, pb = acc ? gw : -1;
                for (int l = 2; l <= L; l++) {
                    if (I.level_size[l] <= 8) {
                        const int offc = I.level_off[l - 1], szc = I.level_size[l - 1];
                        for (int p = 0; p < I.level_size[l]; p++) {
                            const int c = p * 32 + lane;
                            const long long t = c < szc ? NT[offc + c] : SP_INF_BITS;
                            const int i = c < szc ? NI[offc + c] : INT_MAX;
                            long long mt;
                            int mi;
                            argmin_redux(t, i, mt, mi);
                            if (lane == 0) { NT[I.level_off[l] + p] = mt; NI[I.level_off[l] + p] = mi; }
                        }
                        __syncwarp();
                        continue;
                    }
                    pa = pa >= 0 ? pa >> 5 : -1;
                    pb = pb >= 0 ? pb >> 5 : -1;
                    // one lane per distinct parent: the first to raise its flag
                    int* fl = flg + (I.level_off[l] - flg_base);
                    const bool lead_a = pa >= 0 && atomicExch(&fl[pa], 1) == 0;
                    const bool lead_b = pb >= 0 && atomicExch(&fl[pb], 1) == 0;
                    if (lead_a) lane_node(I, NT, NI, l, pa);
                    if (lead_b) lane_node(I, NT, NI, l, pb);
                    __syncwarp();
                    if (lead_a) fl[pa] = 0;
                    if (lead_b) fl[pb] = 0;
                    if (!lead_a) pa = -1;
                    if (!lead_b) pb = -1;
                }
                rt = NT[I.level_off[L]];
                ri = NI[I.level_off[L]];
                if (over) { step_done = true; break; }
                if (status != SP_TRAJ_OK) break;
            }
            if (step_done) step++;
            else break;
        }
        __syncwarp();
        for (int e = lane; e < NN; e += 32) { T.node_t[e] = NT[e]; T.node_i[e] = NI[e]; }
        for (int e = lane; e < N1; e += 32) T.node_t2[e] = T2[e];
        if (lane == 0) {
            T.evn = evn;
            T.nrx = nrx;
            T.ndf = ndf;
            T.step = step;
            T.status = status;
            T.t_last = tlast;
            T.a_tot = A;
            T.bscale = bsc;
            T.nbatch += stat_b;
            T.ncand += stat_c;
            if (errv >= 0) T.err_voxel = errv;
        }
        __syncwarp();
    }
}

typedef void (*BatchFn)(NsmTraj*, const NsmInstance*, int, int, double, long long, long long, int*,
                        const int*);

template <bool REF>
static BatchFn pick_batch(int variant) {
    switch (variant) {
        case 1: return nsm_advance_batch<REF, 4, 8, false>;
        case 2: return nsm_advance_batch<REF, 8, 16, false>;
        case 3: return nsm_advance_batch<REF, 1, 2, true>;
        default: return nsm_advance_batch<REF, 3, 4, true>;
    }
}

void launch_nsm_batch(bool ref, int variant, int warp_smem, NsmTraj* trajs,
                      const NsmInstance* insts, int ntraj, int step_end, double dt,
                      long long budget, long long max_ns, int* work, int num_sms,
                      const int* tlist, cudaStream_t st) {
    cudaMemsetAsync(work, 0, sizeof(int), st);
    const int per_sm = (200 * 1024) / warp_smem > 0 ? (200 * 1024) / warp_smem : 1;
    int blocks = ntraj;
    const int cap = num_sms * (per_sm < 32 ? per_sm : 32);
    if (blocks > cap) blocks = cap;
    BatchFn fn = ref ? pick_batch<true>(variant) : pick_batch<false>(variant);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    fn<<<blocks, 32, warp_smem, st>>>(trajs, insts, ntraj, step_end, dt, budget, max_ns, work,
                                      tlist);
}

}  // namespace spg
