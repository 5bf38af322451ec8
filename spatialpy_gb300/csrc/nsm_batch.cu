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

#include "common.cuh"
#include "nsm_small.cuh"

namespace spg {

constexpr int kFront = 64;

// per-warp shared memory of the batch kernel
int nsm_batch_smem(const NsmInstance& d) {
    size_t b = (size_t)d.num_nodes * 8 + (size_t)d.level_size[1] * 8 + (size_t)d.num_nodes * 4;
    b += 2 * kFront * 4;
    b += (size_t)(d.num_nodes - d.level_size[1]) * 4;   // repair flags, levels >= 2
    return (int)((b + 15) / 16 * 16);
}

// Level-1 nodes with time < thb, into lane-held (ct, ci).  Returns the
// count, or -1 when more than 32 (or a frontier overflow).  Levels above 2
// are walked one frontier node at a time; the level-2 frontier (at most 32
// nodes) is expanded in parallel, one node per lane, its 32 children read
// in a lane-rotated order (no bank conflicts) and selected by bit masks.
__device__ __forceinline__ int batch_extract(const NsmInstance& I, const long long* NT,
                                             const int* NI, int* fa, int* fb, int lane,
                                             unsigned ltm, long long thb, long long& ct,
                                             int& ci) {
    const int L = I.levels;
    int nf = 1;
    if (lane == 0) fa[0] = 0;
    __syncwarp();
    int* cur = fa;
    int* nxt = fb;
    for (int l = L; l >= 3; l--) {
        const int off = I.level_off[l - 1], sz = I.level_size[l - 1];
        int nn = 0;
        for (int f = 0; f < nf; f++) {
            const int c = cur[f] * 32 + lane;
            const long long t = c < sz ? NT[off + c] : SP_INF_BITS;
            const bool q = t < thb;
            const unsigned bal = __ballot_sync(SP_FULL, q);
            const int pos = nn + __popc(bal & ltm);
            if (q && pos < kFront) nxt[pos] = c;
            nn += __popc(bal);
        }
        __syncwarp();
        if (nn > kFront) return -1;
        nf = nn;
        int* tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
    // level 2 -> level 1
    const int off = I.level_off[1], sz = I.level_size[1];
    int got = 0;
    if (nf <= 32) {
        unsigned mask = 0u;
        int base = 0;
        if (lane < nf) {
            base = cur[lane] * 32;
            if ((off & 1) == 0 && base + 32 <= sz) {
                const longlong2* tp = (const longlong2*)(NT + off + base);
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const int qq = (q + lane) & 15;
                    const longlong2 u = tp[qq];
                    mask |= (unsigned)(u.x < thb) << (2 * qq);
                    mask |= (unsigned)(u.y < thb) << (2 * qq + 1);
                }
            } else {
                for (int q = 0; q < 32; q++)
                    if (base + q < sz && NT[off + base + q] < thb) mask |= 1u << q;
            }
        }
        // exclusive prefix of the per-lane counts
        const int n = __popc(mask);
        int inc = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(SP_FULL, inc, o);
            if (lane >= o) inc += u;
        }
        got = __shfl_sync(SP_FULL, inc, 31);
        __syncwarp();
        if (got <= 32) {
            int pos = inc - n;
            for (unsigned m = mask; m; m &= m - 1) nxt[pos++] = base + __ffs(m) - 1;
        }
    } else {
        got = 33;
    }
    __syncwarp();
    if (got > 32) return -1;
    if (lane < got) {
        const int node = nxt[lane];
        ct = NT[off + node];
        ci = NI[off + node];
    } else {
        ct = SP_INF_BITS;
        ci = INT_MAX;
    }
    __syncwarp();
    return got;
}

// ascending bitonic sort of 32 lanes by (t, i)
__device__ __forceinline__ void bitonic32(int lane, long long& ct, int& ci) {
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
            const long long pt = __shfl_xor_sync(SP_FULL, ct, jj);
            const int pi = __shfl_xor_sync(SP_FULL, ci, jj);
            const bool up = (lane & k) == 0;
            const bool lower = (lane & jj) == 0;
            const bool take = (lower == up) ? kless(pt, pi, ct, ci) : kless(ct, ci, pt, pi);
            if (take) {
                ct = pt;
                ci = pi;
            }
        }
    }
}

// One lane: minimum and second minimum of leaf group g (32 contiguous leaf
// times) -> level-1 node g and its second-smallest time.  Two halves of 16
// leaves, each reduced by a pairwise tree (the merges of one level are
// independent, so their latencies overlap), then merged.
struct MinPair {
    long long m, s;   // smallest time (with its index) and the second-smallest time
    int i;
};

__device__ __forceinline__ MinPair merge_pair(const MinPair& a, const MinPair& b) {
    const bool x = kless(a.m, a.i, b.m, b.i);
    MinPair r;
    r.m = x ? a.m : b.m;
    r.i = x ? a.i : b.i;
    const long long hi = x ? b.m : a.m;
    const long long s1 = x ? a.s : b.s;
    r.s = hi < s1 ? hi : s1;
    return r;
}

__device__ __forceinline__ MinPair rescan_half(const longlong2* p, int base) {
    MinPair v[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const longlong2 u = p[q];
        const bool a = u.x <= u.y;               // ties: the lower index wins
        v[q].m = a ? u.x : u.y;
        v[q].i = a ? base + 2 * q : base + 2 * q + 1;
        v[q].s = a ? u.y : u.x;
    }
#pragma unroll
    for (int w = 4; w >= 1; w >>= 1)
#pragma unroll
        for (int q = 0; q < w; q++) v[q] = merge_pair(v[q], v[q + w]);
    return v[0];
}

// groups ga and gb (gb < 0: none), both groups' loads in flight together
__device__ __forceinline__ void lane_rescan2(const NsmInstance& I, const long long* LF,
                                             long long* NT, int* NI, long long* T2, int ga,
                                             int gb) {
    const int gq = gb >= 0 ? gb : ga;
    const longlong2* pa = (const longlong2*)(LF + (size_t)ga * 32);
    const longlong2* pb = (const longlong2*)(LF + (size_t)gq * 32);
    const MinPair a0 = rescan_half(pa, ga * 32), b0 = rescan_half(pb, gq * 32);
    const MinPair a1 = rescan_half(pa + 8, ga * 32 + 16), b1 = rescan_half(pb + 8, gq * 32 + 16);
    const MinPair ra = merge_pair(a0, a1), rb = merge_pair(b0, b1);
    NT[I.level_off[1] + ga] = ra.m;
    NI[I.level_off[1] + ga] = ra.i;
    T2[ga] = ra.s;
    if (gb >= 0) {
        NT[I.level_off[1] + gb] = rb.m;
        NI[I.level_off[1] + gb] = rb.i;
        T2[gb] = rb.s;
    }
}

// One lane: node p of level l (>= 2) from its 32 children, read in an order
// rotated by p so that lanes working on different nodes hit different banks;
// the argmin is a pairwise tree over each half of the children.
__device__ __forceinline__ void lane_node(const NsmInstance& I, long long* NT, int* NI, int l, int p) {
    const int offc = I.level_off[l - 1], szc = I.level_size[l - 1];
    long long bt = SP_INF_BITS;
    int bi = INT_MAX;
    if ((offc & 1) == 0 && p * 32 + 32 <= szc) {
        // full node, 16-byte aligned children: two per load
        const longlong2* tp = (const longlong2*)(NT + offc + p * 32);
        const int2* ip = (const int2*)(NI + offc + p * 32);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            long long t[8];
            int id[8];
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int qq = (h * 8 + q + p) & 15;
                const longlong2 a = tp[qq];
                const int2 b = ip[qq];
                const bool x = kless(a.x, b.x, a.y, b.y);
                t[q] = x ? a.x : a.y;
                id[q] = x ? b.x : b.y;
            }
#pragma unroll
            for (int w = 4; w >= 1; w >>= 1)
#pragma unroll
                for (int q = 0; q < w; q++) {
                    const bool x = kless(t[q], id[q], t[q + w], id[q + w]);
                    t[q] = x ? t[q] : t[q + w];
                    id[q] = x ? id[q] : id[q + w];
                }
            if (kless(t[0], id[0], bt, bi)) { bt = t[0]; bi = id[0]; }
        }
    } else {
        for (int q = 0; q < 32; q++) {
            const int c = p * 32 + ((q + p) & 31);
            if (c < szc) {
                const long long t = NT[offc + c];
                const int i = NI[offc + c];
                if (kless(t, i, bt, bi)) { bt = t; bi = i; }
            }
        }
    }
    NT[I.level_off[l] + p] = bt;
    NI[I.level_off[l] + p] = bi;
}

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
                const int v = act ? ci : 0;
                const double tt = __longlong_as_double(ct);
                int xv[MS], xw[MS];
                float dv[MS], dw[MS];
#pragma unroll
                for (int s = 0; s < MS; s++) {
                    const bool on = act && (EX || s < S);
                    xv[s] = on ? X[(size_t)v * S + s] : 0;
                    dv[s] = on ? I.ddiag[(size_t)v * S + s] : 0.0f;
                    xw[s] = 0;
                    dw[s] = 0.0f;
                }
                const int typev = act ? I.type[v] : 0;
                const float volv = act ? I.vol[v] : 1.0f, ivolv = act ? I.ivol[v] : 1.0f;
                const int cnt = act ? I.nbr_cnt[v] : 0;
                const uint64_t ev = evn + (uint64_t)lane;
                const u32x4 rr = philox4x32_10((uint32_t)ev, (uint32_t)(ev >> 32), 0u, 0u, T.key0, T.key1);
                const float ua = u24(rr.x), ub = u24(rr.y);
                const float e0 = neglog_f(u32f(rr.z));
                float srr, sdr;
                rates_small<MS, MR, EX>(Q, xv, dv, volv, ivolv, typev, srr, sdr);
                const float a0v = srr + sdr;
                const bool rxn = ua * a0v <= srr;                 // :255
                int w = -1, sp = 0, err = 0;
                long long tv = SP_INF_BITS, tw = SP_INF_BITS;
                float dA = 0.0f;
                if (act) {
                    if (rxn) {
                        const float target = REF ? ua * srr : ua * a0v;
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
                        if (re < 0) {
                            err = SP_TRAJ_SELECT_OVERFLOW;
                        } else {
                            for (int q = I.jcN[re]; q < I.jcN[re + 1]; q++) {   // :285-296
                                const int s2 = I.irN[q], d = I.prN[q];
#pragma unroll
                                for (int s = 0; s < MS; s++)
                                    if (s == s2) {
                                        xv[s] += d;
                                        if (xv[s] < 0) err = SP_TRAJ_NEG_COUNT;
                                    }
                            }
                            rates_small<MS, MR, EX>(Q, xv, dv, volv, ivolv, typev, srr, sdr);
                            const float a1v = srr + sdr;
                            tv = draw_time(tt, e0, a1v);
                            dA = a1v - a0v;
                        }
                    } else {
                        const float target = REF ? ua * sdr : ua * a0v - srr;
                        float cum = 0.0f;
                        int sps = -1, last = -1;
#pragma unroll
                        for (int s = 0; s < MS; s++) {            // :319-321
                            if ((EX || s < S) && sps < 0) {
                                const float wgt = dv[s] * (float)xv[s];
                                cum = cum + wgt;
                                if (wgt > 0.0f) {
                                    last = s;
                                    if (target <= cum) sps = s;
                                }
                            }
                        }
                        if (sps < 0) sps = last;
                        if (sps < 0) {
                            err = SP_TRAJ_SELECT_OVERFLOW;
                        } else {
                            sp = sps;
                            const float target2 = ub * pickf<MS>(dv, sp);     // :353-354
                            const int2* crow = I.cdfj + ((size_t)v * S + sp) * K;
                            int k = -1, lastk = -1, jk = -1, jlast = -1;
                            float prev = 0.0f;
                            if (K <= 32 && (K & 1) == 0) {
                                // the whole row in one round (32 entries, 256 bytes,
                                // two per 16-byte load), then the scan of :359-367 as
                                // bit masks: entry q is a candidate when its running
                                // sum rises (positive weight) and a hit when it also
                                // exceeds target2; the first hit, else the last
                                // candidate, is the destination
                                int2 c[32];
                                const int4* crow4 = (const int4*)crow;
#pragma unroll
                                for (int q = 0; q < 16; q++) {
                                    const int4 u = 2 * q < cnt ? crow4[q] : make_int4(0, -1, 0, -1);
                                    c[2 * q] = make_int2(u.x, u.y);
                                    c[2 * q + 1] = make_int2(u.z, u.w);
                                }
                                unsigned posm = 0u, hitm = 0u;
#pragma unroll
                                for (int q = 0; q < 32; q++) {
                                    const float cq = __int_as_float(c[q].x);
                                    const float cp = q == 0 ? 0.0f : __int_as_float(c[q - 1].x);
                                    const bool pos = q < cnt && cq > cp;
                                    posm |= (unsigned)pos << q;
                                    hitm |= (unsigned)(pos && cq > target2) << q;
                                }
                                if (hitm) k = __ffs(hitm) - 1;
                                else if (posm) lastk = 31 - __clz(posm);
                                const int ks = hitm ? k : lastk;
#pragma unroll
                                for (int q = 0; q < 32; q++)
                                    if (q == ks) jk = c[q].y;
                                jlast = jk;
                                (void)prev;
                            } else {
                                for (int q = 0; q < cnt && k < 0; q++) {
                                    const int2 cc = crow[q];
                                    const float cq = __int_as_float(cc.x);
                                    if (cq > prev) {
                                        lastk = q;
                                        jlast = cc.y;
                                        if (cq > target2) { k = q; jk = cc.y; }
                                    }
                                    prev = cq;
                                }
                            }
                            if (k < 0) { k = lastk; jk = jlast; }
                            if (k < 0) {
                                err = SP_TRAJ_SELECT_OVERFLOW;
                            } else {
                                w = jk;
#pragma unroll
                                for (int s = 0; s < MS; s++) {
                                    const bool on = EX || s < S;
                                    xw[s] = on ? X[(size_t)w * S + s] : 0;
                                    dw[s] = on ? I.ddiag[(size_t)w * S + s] : 0.0f;
                                }
                                const int typew = I.type[w];
                                // the engine evaluates the destination's reactions
                                // with the source voxel's volume (:431-433)
                                const float volw = REF ? volv : I.vol[w];
                                const float ivolw = REF ? ivolv : I.ivol[w];
                                rates_small<MS, MR, EX>(Q, xw, dw, volw, ivolw, typew, srr, sdr);
                                const float a0w = srr + sdr;
#pragma unroll
                                for (int s = 0; s < MS; s++)              // :394-402
                                    if (s == sp && w != v) { xv[s] -= 1; xw[s] += 1; }
                                rates_small<MS, MR, EX>(Q, xv, dv, volv, ivolv, typev, srr, sdr);
                                const float a1v = srr + sdr;
                                rates_small<MS, MR, EX>(Q, xw, dw, volw, ivolw, typew, srr, sdr);
                                const float a1w = srr + sdr;
                                const float e1 = neglog_f(u32f(rr.w));
                                tv = draw_time(tt, e0, a1v);
                                tw = draw_time(tt, e1, a1w);
                                dA = (a1v - a0v) + (a1w - a0w);
                            }
                        }
                    }
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
