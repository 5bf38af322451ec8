// nsm_batchw.cu — speculative batched NSM event loop with W warps (one CTA)
// per trajectory: batches of up to 32*W candidates.
//
// The events, their order and their random numbers are those of the
// sequential loop (nsm.cu) and of the one-warp batch kernel (nsm_batch.cu);
// only the work of a batch is spread over more warps, so that one
// trajectory keeps several schedulers of an SM busy:
//
//  1. candidates: warp 0 walks the shared-memory tree down to level 2; the
//     level-2 frontier (up to 32*W nodes) is expanded by all warps, one node
//     per lane, into the leaf groups whose minimum lies below the horizon,
//     and EVERY leaf below the horizon is a candidate (a group's runner-up
//     included).  Each group keeps its two or three smallest leaves (time
//     and voxel) in shared memory, so a group's 32 leaf times are read from
//     global memory only when every leaf of its list lies below the
//     horizon.  The candidates are ordered by (time, voxel): each warp
//     sorts its 32 keys with a bitonic network over shuffles, and a key's
//     rank adds the keys of the other warps below it (binary search of their
//     sorted lists).  Each candidate's counts line is prefetched into L1.
//  2. thread g executes candidate g as event number n+g.
//  3. the accepted prefix: time bounds by prefix minima of the redrawn times
//     (warp shuffles, then the minima of earlier warps); voxel conflicts
//     through a hashed table of the smallest candidate index touching each
//     voxel.  No leaf outside the candidates lies below the horizon, so no
//     group bound cuts the prefix: with group minima as candidates a group's
//     runner-up had to stay above every later candidate, which cut batches
//     near the birthday bound of the 2,000 groups (about 48 events of 128);
//     with leaves only the 64,000 voxels' conflicts and redrawn times do.
//  4. accepted events are written and, after a CTA barrier, each group
//     changed by one event has its list updated in place by that event's
//     thread; a group changed by several events, or whose list falls below
//     two entries, is rescanned from its leaves, 4 lanes per group (8
//     leaves per lane, merged by shuffles) with all loads in flight (a
//     source group likely to need it was prefetched into L1 during the
//     execution).  Then the level-2 nodes above changed group minima,
//     listed before the rescans, are recomputed by 4 lanes each, and
//     warp 0 recomputes the small levels above.
//
// Scalars that steer the loop (clock, counters, running propensity total)
// are kept in every thread and updated from the same shared values in the
// same order, so all warps take the same branches.  Compiled with
// -fmad=false.
#include "nsm_batch.cuh"

namespace spg {

constexpr int kHash = 1024;   // conflict table slots (power of two, >= 4 * 2 * 32 * W)

__device__ __forceinline__ int hslot(int v) { return (int)(((unsigned)v * 2654435761u) >> 22); }

// conflict table: open addressing with linear probing, key = voxel, value =
// the smallest candidate index touching it.  At most 2 * 32 * W keys per
// batch, so a probe always ends at the key or at an empty slot.
__device__ __forceinline__ void ctab_insert(int* key, int* val, int v, int g) {
    int h = hslot(v);
    for (int n = 0; n < kHash; n++) {
        const int old = atomicCAS(&key[h], -1, v);
        if (old == -1 || old == v) {
            atomicMin(&val[h], g);
            return;
        }
        h = (h + 1) & (kHash - 1);
    }
}

__device__ __forceinline__ int ctab_find(const int* key, int v) {
    int h = hslot(v);
    for (int n = 0; n < kHash; n++) {
        if (key[h] == v) return h;
        h = (h + 1) & (kHash - 1);
    }
    return -1;
}

// The three smallest leaves of a group, (time, voxel) in (time, voxel) order.
struct Top3 {
    long long t0, t1, t2;
    int i0, i1, i2;
};

__device__ __forceinline__ Top3 merge3(const Top3& a, const Top3& b) {
    const bool fa = kless(a.t0, a.i0, b.t0, b.i0);
    Top3 r;
    r.t0 = fa ? a.t0 : b.t0;
    r.i0 = fa ? a.i0 : b.i0;
    const long long ha = fa ? a.t1 : a.t0, hb = fa ? b.t0 : b.t1;   // the lists' next heads
    const int hai = fa ? a.i1 : a.i0, hbi = fa ? b.i0 : b.i1;
    const long long na = fa ? a.t2 : a.t1, nb = fa ? b.t1 : b.t2;   // and the items after them
    const int nai = fa ? a.i2 : a.i1, nbi = fa ? b.i1 : b.i2;
    const bool fs = kless(ha, hai, hb, hbi);
    r.t1 = fs ? ha : hb;
    r.i1 = fs ? hai : hbi;
    const long long c1 = fs ? na : ha, c2 = fs ? hb : nb;
    const int c1i = fs ? nai : hai, c2i = fs ? hbi : nbi;
    const bool f3 = kless(c1, c1i, c2, c2i);
    r.t2 = f3 ? c1 : c2;
    r.i2 = f3 ? c1i : c2i;
    return r;
}

// 16 leaves (8 aligned pairs) starting at leaf `base`
__device__ __forceinline__ Top3 top3_half(const longlong2* p, int base) {
    Top3 v[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const longlong2 u = p[q];
        const bool a = u.x <= u.y;               // ties: the lower index first
        v[q].t0 = a ? u.x : u.y;
        v[q].t1 = a ? u.y : u.x;
        v[q].t2 = SP_INF_BITS;
        v[q].i0 = a ? base + 2 * q : base + 2 * q + 1;
        v[q].i1 = a ? base + 2 * q + 1 : base + 2 * q;
        v[q].i2 = INT_MAX;
    }
#pragma unroll
    for (int w = 4; w >= 1; w >>= 1)
#pragma unroll
        for (int q = 0; q < w; q++) v[q] = merge3(v[q], v[q + w]);
    return v[0];
}

// Each group keeps a list of its k smallest leaves, (time, voxel) in order:
// the first is the level-1 node (NT, NI), the second the runner-up (T2, I2;
// the other event kernels keep T2 too), the third (T3, I3).  Every leaf of
// the group outside the list has a larger key than the list's last entry.
// KC holds k in its low byte; between batches k is 2 or 3.

// The full list (k = 3) of group g from its 32 leaf times.
__device__ __forceinline__ void rescan3(const NsmInstance& I, const long long* LF, long long* NT,
                                        int* NI, long long* T2, int* I2, long long* T3, int* I3,
                                        int* KC, int g) {
    const longlong2* p = (const longlong2*)(LF + (size_t)g * 32);
    const Top3 a = top3_half(p, g * 32);
    const Top3 b = top3_half(p + 8, g * 32 + 16);
    const Top3 r = merge3(a, b);
    NT[I.level_off[1] + g] = r.t0;
    NI[I.level_off[1] + g] = r.i0;
    T2[g] = r.t1;
    I2[g] = r.i1;
    T3[g] = r.t2;
    I3[g] = r.i2;
    KC[g] = 3;
}

// Group g's list after voxel vn's leaf time became tn, without reading the
// leaves: vn leaves the list if it was in it, and enters it when its new
// key is below the old last entry (the entry then dropped, if the list was
// full, is the largest of the four).  Returns the new k; the list stays
// exact, but below 2 entries the group must be rescanned.  N1t, N1i point
// at level 1 of the tree.
__device__ __forceinline__ int list_update(long long* N1t, int* N1i, long long* T2, int* I2,
                                           long long* T3, int* I3, int g, int k, long long tn,
                                           int vn) {
    long long t[3] = {N1t[g], T2[g], T3[g]};
    int i[3] = {N1i[g], I2[g], I3[g]};
    const long long Mt = k >= 3 ? t[2] : k == 2 ? t[1] : t[0];
    const int Mi = k >= 3 ? i[2] : k == 2 ? i[1] : i[0];
    const bool ins = k > 0 && kless(tn, vn, Mt, Mi);
    int p = -1;
#pragma unroll
    for (int q = 0; q < 3; q++)
        if (q < k && i[q] == vn) p = q;
    if (p >= 0) {
#pragma unroll
        for (int q = 0; q < 2; q++)
            if (q >= p && q + 1 < k) { t[q] = t[q + 1]; i[q] = i[q + 1]; }
        k--;
    } else if (ins && k == 3) {
        k = 2;
    }
    if (ins) {
        int pos = 0;
#pragma unroll
        for (int q = 0; q < 3; q++)
            if (q < k && kless(t[q], i[q], tn, vn)) pos++;
#pragma unroll
        for (int q = 2; q >= 1; q--)
            if (q <= k && q > pos) { t[q] = t[q - 1]; i[q] = i[q - 1]; }
#pragma unroll
        for (int q = 0; q < 3; q++)
            if (q == pos) { t[q] = tn; i[q] = vn; }
        k++;
    }
#pragma unroll
    for (int q = 0; q < 3; q++)
        if (q >= k) { t[q] = SP_INF_BITS; i[q] = INT_MAX; }
    N1t[g] = t[0];
    N1i[g] = i[0];
    T2[g] = t[1];
    I2[g] = i[1];
    T3[g] = t[2];
    I3[g] = i[2];
    return k;
}

// Top3 of two adjacent leaves `base`, `base` + 1
__device__ __forceinline__ Top3 pair3(const longlong2 u, int base) {
    const bool a = u.x <= u.y;                   // ties: the lower index first
    Top3 r;
    r.t0 = a ? u.x : u.y;
    r.t1 = a ? u.y : u.x;
    r.t2 = SP_INF_BITS;
    r.i0 = a ? base : base + 1;
    r.i1 = a ? base + 1 : base;
    r.i2 = INT_MAX;
    return r;
}

__device__ __forceinline__ Top3 shfl_xor3(const Top3& t, int o) {
    Top3 q;
    q.t0 = __shfl_xor_sync(SP_FULL, t.t0, o);
    q.t1 = __shfl_xor_sync(SP_FULL, t.t1, o);
    q.t2 = __shfl_xor_sync(SP_FULL, t.t2, o);
    q.i0 = __shfl_xor_sync(SP_FULL, t.i0, o);
    q.i1 = __shfl_xor_sync(SP_FULL, t.i1, o);
    q.i2 = __shfl_xor_sync(SP_FULL, t.i2, o);
    return q;
}

static size_t batchw_smem_bytes(const NsmInstance& d, int W) {
    const size_t NN = d.num_nodes, N1 = d.level_size[1];
    size_t b = NN * 8 + N1 * 8 + NN * 4;      // tree times, second minima, indices
    b += N1 * 20;                              // third minima, runner-up and third voxels, k
    b += 2 * (size_t)(64 * W) * 4;             // frontiers
    b += (NN - N1) * 4;                        // repair flags, levels >= 2
    b += (size_t)kHash * 8;                    // conflict table: keys, values
    b += (size_t)(32 * W) * 4;                 // candidate groups
    b = (b + 15) / 16 * 16;
    b += 2 * (size_t)(32 * W) * 12;            // sort exchange, double-buffered
    b += (size_t)(32 * W) * 12;                // candidate leaves: times, voxels
    return (b + 15) / 16 * 16;
}

int nsm_batchw_smem(const NsmInstance& d, int W) { return (int)batchw_smem_bytes(d, W); }

template <bool REF, int MS, int MR, bool EX, int W>
__global__ void __launch_bounds__(32 * W, 1)
    nsm_advance_batchw(NsmTraj* trajs, const NsmInstance* insts, int ntraj, int step_end,
                       double dt, long long budget, long long max_ns, int* work,
                       const int* tlist) {
    constexpr int NC = 32 * W;    // candidates per batch at most
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_jt, s_nf, s_tflag, s_nr, s_nl;
    __shared__ int s_wcnt[W], s_wfi[W], s_werr[W], s_werrc[W], s_werrv[W], s_wnrx[W], s_wndf[W];
    __shared__ long long s_wmin[W], s_tl;
    __shared__ double s_wdA[W];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const unsigned ltm = (1u << lane) - 1u;
    for (;;) {
        if (tid == 0) s_jt = atomicAdd(work, 1);
        __syncthreads();
        const int jt = s_jt;
        __syncthreads();
        if (jt >= ntraj) return;
        NsmTraj& T = trajs[tlist ? tlist[jt] : jt];
        if (T.status != SP_TRAJ_OK || T.step >= step_end) continue;
        const NsmInstance& I = insts[T.inst];
        const int NN = I.num_nodes, N1 = I.level_size[1], L = I.levels;
        SmallNet<MS, MR> Q;
        Q.S = I.S;
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
        // shared-memory layout (batchw_smem_bytes)
        long long* NT = (long long*)smem;
        long long* T2 = NT + NN;
        long long* T3 = T2 + N1;                   // third-smallest leaf time per group
        int* NI = (int*)(T3 + N1);
        int* I2 = NI + NN;                         // runner-up voxel per group
        int* I3 = I2 + N1;                         // third voxel per group
        int* KC = I3 + N1;                         // list length k | changes << 8
        int* fa = KC + N1;
        int* fb = fa + 64 * W;
        int* flg = fb + 64 * W;
        int* hkey = flg + (NN - N1);
        int* hval = hkey + kHash;
        int* clist = hval + kHash;
        unsigned char* xb = (unsigned char*)(((uintptr_t)(clist + NC) + 15) & ~(uintptr_t)15);
        long long* xt = (long long*)xb;            // [2][NC]
        int* xi = (int*)(xt + 2 * NC);             // [2][NC]
        long long* lt = (long long*)(xi + 2 * NC); // [NC] candidate leaf times
        int* lv = (int*)(lt + NC);                 // [NC] candidate voxels
        const int flg_base = I.level_off[2];
        for (int e = tid; e < NN - N1; e += NC) flg[e] = 0;
        for (int e = tid; e < kHash; e += NC) { hkey[e] = -1; hval[e] = INT_MAX; }
        for (int e = tid; e < NN; e += NC) { NT[e] = T.node_t[e]; NI[e] = T.node_i[e]; }
        __syncthreads();
        // level 1 with the groups' lists from the leaves (the other event
        // kernels keep only the runner-up times)
        for (int g = tid; g < N1; g += NC) rescan3(I, T.leaf, NT, NI, T2, I2, T3, I3, KC, g);
        __syncthreads();
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
                    // one thread reads the clock; every thread takes its answer
                    if (tid == 0) {
                        unsigned long long now;
                        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
                        s_tflag = (long long)(now - t_start) > max_ns;
                    }
                    __syncthreads();
                    const int tf = s_tflag;
                    __syncthreads();
                    if (tf) { status = SP_TRAJ_BUDGET_EXHAUSTED; break; }
                }
                // ---- 1. candidates -------------------------------------------
                if (tid == 0) { s_nr = 0; s_nl = 0; }   // list lengths of step 5
                long long ct = SP_INF_BITS, ct2 = SP_INF_BITS;
                int ci = INT_MAX, count = 1;
                if (over) {   // the reference's one event past the step end, alone
                    if (tid == 0) { ct = rt; ci = ri; ct2 = T2[ri >> 5]; }
                } else {
                    float delta = A > 0.0 ? bsc / (float)A : 3.0e38f;
                    if (!(delta > 0.0f)) delta = 3.0e38f;
                    const double th = __longlong_as_double(rt) + (double)delta;
                    long long thb = __double_as_longlong(th);
                    if (thb > t_end_bits + 1) thb = t_end_bits + 1;   // no event past t_end
                    if (thb <= rt) thb = rt + 1;
                    // levels L..3 by warp 0: frontier of level-2 nodes in fa
                    if (wid == 0) {
                        int nf = 1;
                        if (lane == 0) fa[0] = 0;
                        __syncwarp();
                        int* cur = fa;
                        int* nxt = fb;
                        for (int l = L; l >= 3 && nf >= 0; l--) {
                            const int off = I.level_off[l - 1], sz = I.level_size[l - 1];
                            int nn = 0;
                            for (int f = 0; f < nf; f++) {
                                const int c = cur[f] * 32 + lane;
                                const long long t = c < sz ? NT[off + c] : SP_INF_BITS;
                                const bool q = t < thb;
                                const unsigned bal = __ballot_sync(SP_FULL, q);
                                const int pos = nn + __popc(bal & ltm);
                                if (q && pos < 64 * W) nxt[pos] = c;
                                nn += __popc(bal);
                            }
                            __syncwarp();
                            nf = nn > 64 * W ? -1 : nn;
                            int* tmp = cur;
                            cur = nxt;
                            nxt = tmp;
                        }
                        if (nf > 0 && cur != fa)
                            for (int e = lane; e < nf; e += 32) fa[e] = cur[e];
                        if (lane == 0) s_nf = nf > NC ? -1 : nf;
                    }
                    __syncthreads();
                    const int nf = s_nf;
                    // level 2 -> level 1: frontier node `tid` per thread
                    const int off1 = I.level_off[1], sz1 = I.level_size[1];
                    unsigned mask = 0u;
                    int base = 0;
                    if (nf > 0 && tid < nf) {
                        base = fa[tid] * 32;
                        if ((off1 & 1) == 0 && base + 32 <= sz1) {
                            const longlong2* tp = (const longlong2*)(NT + off1 + base);
#pragma unroll
                            for (int q = 0; q < 16; q++) {
                                const int qq = (q + lane) & 15;
                                const longlong2 u = tp[qq];
                                mask |= (unsigned)(u.x < thb) << (2 * qq);
                                mask |= (unsigned)(u.y < thb) << (2 * qq + 1);
                            }
                        } else {
                            for (int q = 0; q < 32; q++)
                                if (base + q < sz1 && NT[off1 + base + q] < thb) mask |= 1u << q;
                        }
                    }
                    const int n = __popc(mask);
                    int inc = n;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int u = __shfl_up_sync(SP_FULL, inc, o);
                        if (lane >= o) inc += u;
                    }
                    if (lane == 31) s_wcnt[wid] = inc;
                    __syncthreads();
                    int wbase = 0, got = 0;
#pragma unroll
                    for (int u = 0; u < W; u++) {
                        if (u < wid) wbase += s_wcnt[u];
                        got += s_wcnt[u];
                    }
                    if (nf < 0) got = NC + 1;
                    if (got <= NC) {
                        int pos = wbase + inc - n;
                        for (unsigned m = mask; m; m &= m - 1) clist[pos++] = base + __ffs(m) - 1;
                    }
                    __syncthreads();
                    // level 1 -> leaves: group clist[tid] per thread.  Its
                    // minimum is below the horizon; its runner-up too when
                    // T2 < horizon; only when the list's last entry lies
                    // below the horizon are its 32 leaf times read (16-byte
                    // loads; padded leaves hold infinity)
                    int lgot = NC + 1;
                    if (got <= NC) {
                        unsigned lm = 0u;
                        int gb = 0, g = -1, nl = 0;
                        bool scan = false;
                        if (tid < got) {
                            g = clist[tid];
                            gb = g * 32;
                            const bool k3 = (KC[g] & 255) == 3;   // else k = 2
                            if ((k3 ? T3[g] : T2[g]) < thb) {
                                scan = true;
                                const longlong2* lp = (const longlong2*)(LF + gb);
#pragma unroll
                                for (int q = 0; q < 16; q++) {
                                    const longlong2 u = lp[q];
                                    lm |= (unsigned)(u.x < thb) << (2 * q);
                                    lm |= (unsigned)(u.y < thb) << (2 * q + 1);
                                }
                                nl = __popc(lm);
                            } else {
                                nl = k3 && T2[g] < thb ? 2 : 1;
                            }
                        }
                        int li = nl;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) {
                            const int u = __shfl_up_sync(SP_FULL, li, o);
                            if (lane >= o) li += u;
                        }
                        if (lane == 31) s_wcnt[wid] = li;
                        __syncthreads();
                        int lbase = 0;
                        lgot = 0;
#pragma unroll
                        for (int u = 0; u < W; u++) {
                            if (u < wid) lbase += s_wcnt[u];
                            lgot += s_wcnt[u];
                        }
                        if (lgot <= NC && tid < got) {
                            int pos = lbase + li - nl;
                            if (scan) {
                                for (unsigned m = lm; m; m &= m - 1) {
                                    const int e = gb + __ffs(m) - 1;
                                    lt[pos] = LF[e];
                                    lv[pos] = e;
                                    pos++;
                                }
                            } else {
                                lt[pos] = NT[off1 + g];
                                lv[pos] = NI[off1 + g];
                                if (nl == 2) {
                                    lt[pos + 1] = T2[g];
                                    lv[pos + 1] = I2[g];
                                }
                            }
                        }
                        __syncthreads();
                    }
                    if (lgot > NC) {
                        if (bsc > 1.0f) { bsc *= 0.5f; continue; }
                        count = 1;        // degenerate: the minimum alone
                        ct = tid == 0 ? rt : SP_INF_BITS;
                        ci = tid == 0 ? ri : INT_MAX;
                    } else {
                        count = lgot;
                        // order by (time, voxel); keys are distinct (one per
                        // voxel).  Each warp sorts its 32 keys with a bitonic
                        // network over shuffles (padding keys sort last); a
                        // key's rank is its place in its warp plus the keys
                        // of the other warps below it, found by binary search
                        // of their sorted lists.
                        long long kt = SP_INF_BITS;
                        int ki = INT_MAX;
                        if (tid < count) {
                            kt = lt[tid];
                            ki = lv[tid];
                            // the candidate's counts, read first by its
                            // execution: start bringing the line into L1
                            asm volatile("prefetch.global.L1 [%0];" ::"l"(X + (size_t)ki * Q.S));
                        }
#pragma unroll
                        for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
                            for (int j = k >> 1; j > 0; j >>= 1) {
                                const long long pt = __shfl_xor_sync(SP_FULL, kt, j);
                                const int pi = __shfl_xor_sync(SP_FULL, ki, j);
                                // the lower index of an ascending pair keeps the
                                // smaller key, of a descending pair the larger
                                const bool keep_min = ((lane & j) == 0) == ((lane & k) == 0);
                                if (kless(pt, pi, kt, ki) == keep_min) {
                                    kt = pt;
                                    ki = pi;
                                }
                            }
                        }
                        xt[tid] = kt;          // warp wid's sorted keys at [32 wid, 32 wid + 32)
                        xi[tid] = ki;
                        __syncthreads();
                        int rank = lane;
#pragma unroll
                        for (int u = 0; u < W; u++) {
                            if (u == wid) continue;
                            const long long* Lt = xt + 32 * u;
                            const int* Li = xi + 32 * u;
                            int pos = 0;
#pragma unroll
                            for (int st2 = 16; st2 >= 1; st2 >>= 1)
                                if (kless(Lt[pos + st2 - 1], Li[pos + st2 - 1], kt, ki)) pos += st2;
                            if (kless(Lt[pos], Li[pos], kt, ki)) pos++;
                            rank += pos;
                        }
                        if (ki != INT_MAX) {
                            xt[NC + rank] = kt;
                            xi[NC + rank] = ki;
                        }
                        __syncthreads();
                        if (tid < count) {
                            ct = xt[NC + tid];
                            ci = xi[NC + tid];
                        }
                    }
                    // every leaf below the horizon is a candidate: no group bound
                    ct2 = SP_INF_BITS;
                    if (count >= 30 * W) bsc = bsc * 0.8f;
                    else if (count < 24 * W && bsc < 64.0f * W) bsc = bsc * 1.25f;
                }
                stat_b++;
                stat_c += count;
                // ---- 2. speculative execution, one candidate per thread -------
                const bool act = tid < count;
                if (act && (KC[ci >> 5] & 255) == 2) {
                    // the source's leaf group, whose list the event will likely
                    // leave at one entry, so that the group is rescanned after
                    // the commit: start bringing its two lines into L1 now
                    const long long* gp = LF + (size_t)(ci >> 5) * 32;
                    asm volatile("prefetch.global.L1 [%0];" ::"l"(gp));
                    asm volatile("prefetch.global.L1 [%0];" ::"l"(gp + 16));
                }
                Cand<MS> Cd;
                batch_execute<REF, MS, MR, EX>(I, Q, X, act, ci, ct, evn + (uint64_t)tid, T.key0,
                                               T.key1, Cd);
                const int v = Cd.v, w = Cd.w, sp = Cd.sp, err = Cd.err;
                // ---- 3. the accepted prefix ------------------------------------
                long long bound = act ? ct2 : SP_INF_BITS;
                if (Cd.tv < bound) bound = Cd.tv;
                if (Cd.tw < bound) bound = Cd.tw;
                long long pm = bound;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const long long u = __shfl_up_sync(SP_FULL, pm, o);
                    if (lane >= o && u < pm) pm = u;
                }
                long long ex = __shfl_up_sync(SP_FULL, pm, 1);
                if (lane == 0) ex = SP_INF_BITS;
                if (lane == 31) s_wmin[wid] = pm;
                if (act) {
                    ctab_insert(hkey, hval, v, tid);
                    if (w >= 0 && w != v) ctab_insert(hkey, hval, w, tid);
                }
                __syncthreads();
#pragma unroll
                for (int u = 0; u < W; u++)
                    if (u < wid && s_wmin[u] < ex) ex = s_wmin[u];
                // an earlier candidate touching v or w (the same rule as the
                // one-warp kernel: two candidates never share a source voxel)
                const int hv = act ? ctab_find(hkey, v) : -1;
                const int hw = act && w >= 0 ? ctab_find(hkey, w) : -1;
                const bool conf = act && ((hv >= 0 && hval[hv] < tid) || (hw >= 0 && hval[hw] < tid));
                const bool valid = act && ct < ex && !conf && (nev + tid) < budget;
                const unsigned vb = __ballot_sync(SP_FULL, valid);
                const unsigned ebits = __ballot_sync(SP_FULL, act && err != 0);
                if (lane == 0) {
                    s_wfi[wid] = vb == SP_FULL ? 32 : __ffs(~vb) - 1;
                    s_werr[wid] = ebits ? __ffs(ebits) - 1 : 32;
                }
                if (ebits && lane == __ffs(ebits) - 1) {
                    s_werrc[wid] = err;
                    s_werrv[wid] = v;
                }
                __syncthreads();
                int m = NC;
#pragma unroll
                for (int u = W - 1; u >= 0; u--)
                    if (s_wfi[u] < 32) m = 32 * u + s_wfi[u];
                int me = NC, mu = -1;
#pragma unroll
                for (int u = W - 1; u >= 0; u--)
                    if (s_werr[u] < 32) { me = 32 * u + s_werr[u]; mu = u; }
                if (me < m) {
                    status = s_werrc[mu];
                    errv = s_werrv[mu];
                    m = me;
                }
                if (hv >= 0) { hkey[hv] = -1; hval[hv] = INT_MAX; }   // read by all: clear
                if (hw >= 0) { hkey[hw] = -1; hval[hw] = INT_MAX; }
                // ---- 4. commit --------------------------------------------------
                const bool acc = tid < m;
                if (acc) {
#pragma unroll
                    for (int s = 0; s < MS; s++)
                        if (EX || s < Q.S) X[(size_t)v * Q.S + s] = Cd.xv[s];
                    LF[v] = Cd.tv;
                    if (w >= 0) {
#pragma unroll
                        for (int s = 0; s < MS; s++)
                            if (s == sp) X[(size_t)w * Q.S + s] = Cd.xw[s];
                        LF[w] = Cd.tw;
                    }
                }
                const int wr = __popc(__ballot_sync(SP_FULL, acc && Cd.rxn));
                const int wd = __popc(__ballot_sync(SP_FULL, acc && !Cd.rxn));
                double dsum = acc ? (double)Cd.dA : 0.0;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) dsum += __shfl_xor_sync(SP_FULL, dsum, o);
                if (lane == 0) {
                    s_wnrx[wid] = wr;
                    s_wndf[wid] = wd;
                    s_wdA[wid] = dsum;
                }
                if (m > 0 && tid == m - 1) s_tl = ct;
                // ---- 5. rescan and tree repair ------------------------------------
                const int off1r = I.level_off[1];
                const int gv = v >> 5;
                const int gw = (w >= 0 && (w >> 5) != gv) ? w >> 5 : -1;
                // the accepted events' changes per group: a group changed by
                // one event is updated in place by that event's thread, a
                // group changed by several is rescanned, and so is a group
                // whose list falls below two entries
                if (acc) {
                    atomicAdd(&KC[gv], 256);
                    if (gw >= 0) atomicAdd(&KC[gw], 256);
                }
                // a group may hold several accepted events: every commit and
                // count is stored before any rescan reads the group
                __syncthreads();
                bool need_a = false, need_b = false, ch_a = false, ch_b = false;
                if (acc) {
                    long long* N1t = NT + off1r;
                    int* N1i = NI + off1r;
                    const int ca = atomicAnd(&KC[gv], 255);   // the first to ask takes the group
                    if (ca >= 512) {
                        need_a = ch_a = true;
                    } else if (ca >= 256) {
                        const long long m0 = N1t[gv];
                        const int m0i = N1i[gv];
                        int k = list_update(N1t, N1i, T2, I2, T3, I3, gv, ca & 255, Cd.tv, v);
                        if (w >= 0 && gw < 0)
                            k = list_update(N1t, N1i, T2, I2, T3, I3, gv, k, Cd.tw, w);
                        KC[gv] = k;
                        need_a = k < 2;
                        ch_a = need_a || N1t[gv] != m0 || N1i[gv] != m0i;
                    }
                    if (gw >= 0) {
                        const int cb = atomicAnd(&KC[gw], 255);
                        if (cb >= 512) {
                            need_b = ch_b = true;
                        } else if (cb >= 256) {
                            const long long m0 = N1t[gw];
                            const int m0i = N1i[gw];
                            const int k =
                                list_update(N1t, N1i, T2, I2, T3, I3, gw, cb & 255, Cd.tw, w);
                            KC[gw] = k;
                            need_b = k < 2;
                            ch_b = need_b || N1t[gw] != m0 || N1i[gw] != m0i;
                        }
                    }
                }
                // the level-2 parents of groups whose minimum changed, one
                // leader each, listed in fb while the groups to rescan are
                // listed in fa (both free after the walk; any order)
                const bool big2 = L >= 2 && I.level_size[2] > 8;
                int* fl2 = flg + (I.level_off[2] - flg_base);
                const int p2a = ch_a ? gv >> 5 : -1, p2b = ch_b ? gw >> 5 : -1;
                const bool lead_a = big2 && p2a >= 0 && atomicExch(&fl2[p2a], 1) == 0;
                const bool lead_b = big2 && p2b >= 0 && atomicExch(&fl2[p2b], 1) == 0;
                if (lead_a) fb[atomicAdd(&s_nl, 1)] = p2a;
                if (lead_b) fb[atomicAdd(&s_nl, 1)] = p2b;
                if (need_a) fa[atomicAdd(&s_nr, 1)] = gv;
                if (need_b) fa[atomicAdd(&s_nr, 1)] = gw;
                __syncthreads();
                if (lead_a) fl2[p2a] = 0;    // elections are over until the next batch
                if (lead_b) fl2[p2b] = 0;
                {
                    const int rtot = s_nr;
                    // 4 lanes per group (lane l4 reads leaves 8*l4 .. 8*l4+7),
                    // two rounds of NC/4 groups with all their loads in flight
                    const int sg = tid >> 2, l4 = tid & 3;
                    for (int r0 = 0; r0 < rtot; r0 += NC / 2) {
                        const int ra = r0 + sg, rb = ra + NC / 4;
                        const int ga = ra < rtot ? fa[ra] : -1;
                        const int gb2 = rb < rtot ? fa[rb] : -1;
                        longlong2 ua[4], ub[4];
                        const int basea = (ga >= 0 ? ga : 0) * 32 + l4 * 8;
                        const int baseb = (gb2 >= 0 ? gb2 : 0) * 32 + l4 * 8;
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            ua[q] = ga >= 0 ? ((const longlong2*)(LF + basea))[q]
                                            : make_longlong2(SP_INF_BITS, SP_INF_BITS);
                            ub[q] = gb2 >= 0 ? ((const longlong2*)(LF + baseb))[q]
                                             : make_longlong2(SP_INF_BITS, SP_INF_BITS);
                        }
                        Top3 ta = merge3(merge3(pair3(ua[0], basea), pair3(ua[1], basea + 2)),
                                         merge3(pair3(ua[2], basea + 4), pair3(ua[3], basea + 6)));
                        Top3 tb = merge3(merge3(pair3(ub[0], baseb), pair3(ub[1], baseb + 2)),
                                         merge3(pair3(ub[2], baseb + 4), pair3(ub[3], baseb + 6)));
#pragma unroll
                        for (int o = 1; o < 4; o <<= 1) {
                            ta = merge3(ta, shfl_xor3(ta, o));
                            tb = merge3(tb, shfl_xor3(tb, o));
                        }
                        if (l4 == 0 && ga >= 0) {
                            NT[off1r + ga] = ta.t0;
                            NI[off1r + ga] = ta.i0;
                            T2[ga] = ta.t1;
                            I2[ga] = ta.i1;
                            T3[ga] = ta.t2;
                            I3[ga] = ta.i2;
                            KC[ga] = 3;
                        }
                        if (l4 == 0 && gb2 >= 0) {
                            NT[off1r + gb2] = tb.t0;
                            NI[off1r + gb2] = tb.i0;
                            T2[gb2] = tb.t1;
                            I2[gb2] = tb.i1;
                            T3[gb2] = tb.t2;
                            I3[gb2] = tb.i2;
                            KC[gb2] = 3;
                        }
                    }
                }
                __syncthreads();
#pragma unroll
                for (int u = 0; u < W; u++) {
                    nrx += s_wnrx[u];
                    ndf += s_wndf[u];
                    A += s_wdA[u];
                }
                evn += (uint64_t)m;
                nev += m;
                if (m > 0) tlast = __longlong_as_double(s_tl);
                if (big2) {
                    // the listed level-2 nodes recomputed by 4 lanes each (8
                    // children per lane, merged by shuffles)
                    const int ltot = s_nl;
                    const int offc = I.level_off[1], szc = I.level_size[1];
                    const int sg = tid >> 2, l4 = tid & 3;
                    for (int r0 = 0; r0 < ltot; r0 += NC / 4) {
                        const int node = r0 + sg < ltot ? fb[r0 + sg] : -1;
                        const int c0 = (node >= 0 ? node : 0) * 32 + 8 * l4;
                        long long t8[8];
                        int i8[8];
#pragma unroll
                        for (int q = 0; q < 8; q++) {
                            const bool ok = node >= 0 && c0 + q < szc;
                            t8[q] = ok ? NT[offc + c0 + q] : SP_INF_BITS;
                            i8[q] = ok ? NI[offc + c0 + q] : INT_MAX;
                        }
#pragma unroll
                        for (int w2 = 4; w2 >= 1; w2 >>= 1)
#pragma unroll
                            for (int q = 0; q < w2; q++)
                                if (kless(t8[q + w2], i8[q + w2], t8[q], i8[q])) {
                                    t8[q] = t8[q + w2];
                                    i8[q] = i8[q + w2];
                                }
#pragma unroll
                        for (int o = 1; o < 4; o <<= 1) {
                            const long long ot = __shfl_xor_sync(SP_FULL, t8[0], o);
                            const int oi = __shfl_xor_sync(SP_FULL, i8[0], o);
                            if (kless(ot, oi, t8[0], i8[0])) {
                                t8[0] = ot;
                                i8[0] = oi;
                            }
                        }
                        if (l4 == 0 && node >= 0) {
                            NT[I.level_off[2] + node] = t8[0];
                            NI[I.level_off[2] + node] = i8[0];
                        }
                    }
                    __syncthreads();
                }
                // the levels above (at most 8 nodes each within the shared
                // memory this kernel takes; any size stays correct): warp 0
                // recomputes every node, one CTA barrier for all of them
                {
                    const int l0 = big2 ? 3 : 2;
                    if (wid == 0) {
                        for (int l2 = l0; l2 <= L; l2++) {
                            const int offc = I.level_off[l2 - 1], szc = I.level_size[l2 - 1];
                            for (int p = 0; p < I.level_size[l2]; p++) {
                                const int c = p * 32 + lane;
                                const long long t = c < szc ? NT[offc + c] : SP_INF_BITS;
                                const int i = c < szc ? NI[offc + c] : INT_MAX;
                                long long mt;
                                int mi;
                                argmin_redux(t, i, mt, mi);
                                if (lane == 0) {
                                    NT[I.level_off[l2] + p] = mt;
                                    NI[I.level_off[l2] + p] = mi;
                                }
                            }
                            __syncwarp();
                        }
                    }
                    __syncthreads();
                }
                rt = NT[I.level_off[L]];
                ri = NI[I.level_off[L]];
                if (over) { step_done = true; break; }
                if (status != SP_TRAJ_OK) break;
            }
            if (step_done) step++;
            else break;
        }
        __syncthreads();
        for (int e = tid; e < NN; e += NC) { T.node_t[e] = NT[e]; T.node_i[e] = NI[e]; }
        for (int e = tid; e < N1; e += NC) T.node_t2[e] = T2[e];
        if (tid == 0) {
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
        __syncthreads();
    }
}

typedef void (*BatchWFn)(NsmTraj*, const NsmInstance*, int, int, double, long long, long long,
                         int*, const int*);

template <bool REF, int W>
static BatchWFn pick_batchw(int variant) {
    switch (variant) {
        case 1: return nsm_advance_batchw<REF, 4, 8, false, W>;
        case 2: return nsm_advance_batchw<REF, 8, 16, false, W>;
        case 3: return nsm_advance_batchw<REF, 1, 2, true, W>;
        default: return nsm_advance_batchw<REF, 3, 4, true, W>;
    }
}

// warps: 2 or 4 per trajectory
void launch_nsm_batchw(bool ref, int variant, int warps, int smem_bytes, NsmTraj* trajs,
                       const NsmInstance* insts, int ntraj, int step_end, double dt,
                       long long budget, long long max_ns, int* work, int num_sms,
                       const int* tlist, cudaStream_t st) {
    cudaMemsetAsync(work, 0, sizeof(int), st);
    const int per_sm = (200 * 1024) / smem_bytes > 0 ? (200 * 1024) / smem_bytes : 1;
    int blocks = ntraj;
    const int cap = num_sms * (per_sm < 16 ? per_sm : 16);
    if (blocks > cap) blocks = cap;
    BatchWFn fn = warps == 4 ? (ref ? pick_batchw<true, 4>(variant) : pick_batchw<false, 4>(variant))
                             : (ref ? pick_batchw<true, 2>(variant) : pick_batchw<false, 2>(variant));
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
    fn<<<blocks, 32 * warps, smem_bytes, st>>>(trajs, insts, ntraj, step_end, dt, budget, max_ns,
                                               work, tlist);
}

}  // namespace spg
