// nsm_batch.cuh — device helpers shared by the speculative batch event
// kernels (nsm_batch.cu: one warp per trajectory; nsm_batchw.cu: several
// warps per trajectory): candidate extraction, sorting, one candidate's
// event, group rescans and tree repair.
#pragma once
#include <climits>
#include <cstdint>

#include "common.cuh"
#include "nsm_small.cuh"

namespace spg {

constexpr int kFront = 64;

// per-warp shared memory of the batch kernel
inline int nsm_batch_smem_w1(const NsmInstance& d) {
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

// ---------------------------------------------------------------------------
// one speculative candidate (lane-parallel): the event at voxel ci at time ct
// as the trajectory's event number ev (Philox counter), in the sequential
// loop's arithmetic.  Outputs: new counts of v (and w), redrawn times,
// the change of the voxels' total propensity, and an error status.
// ---------------------------------------------------------------------------
template <int MS>
struct Cand {
    int v, w, sp, err;
    bool rxn;
    long long tv, tw;
    float dA;
    int xv[MS], xw[MS];
};

template <bool REF, int MS, int MR, bool EX>
__device__ __forceinline__ void batch_execute(const NsmInstance& I, const SmallNet<MS, MR>& Q,
                                              const int32_t* X, bool act, int ci, long long ct,
                                              uint64_t ev, uint32_t key0, uint32_t key1,
                                              Cand<MS>& C) {
    const int S = I.S, K = I.K;
    const int v = act ? ci : 0;
    C.v = v;
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
    const u32x4 rr = philox4x32_10((uint32_t)ev, (uint32_t)(ev >> 32), 0u, 0u, key0, key1);
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
    C.w = w;
    C.sp = sp;
    C.err = err;
    C.rxn = rxn;
    C.tv = tv;
    C.tw = tw;
    C.dA = dA;
#pragma unroll
    for (int s = 0; s < MS; s++) {
        C.xv[s] = xv[s];
        C.xw[s] = xw[s];
    }
}

}  // namespace spg
