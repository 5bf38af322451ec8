// sdpd.cu — SDPD particle step on the GPU (FP32 or FP64).
//
// Restates one engine step of a moving domain (src/simulate_threads.cpp:232-281
// with the kd-tree of :80-108): take_step1 (src/simulate.cpp:56-109),
// find_neighbors + pairwiseForce (particle.cpp:240-294, model.cpp:39-191),
// take_step2 with filterDensity and the boundary volume fraction
// (simulate.cpp:132-173, model.cpp:194-329).  Per step, five launches
// (replayed from a CUDA graph in blocks of 20 steps):
//
//   begin     the predictor, then the cell of each particle's start-of-step
//             position (the kd-tree points of the step) and its rank in that
//             cell (atomic histogram)
//   scan      exclusive scan of the cell counts into cell starts, one CTA
//             per tile of cells offset by the tile totals begin counted; the
//             counts are reset for the next step
//   scatter   counting-sort scatter into cell-ordered, float4-packed copies
//             of what the force pass reads: tree point (+ particle index),
//             current position (+ mass), velocity, transport velocity and
//             {rho, P/rho^2, m/rho, nu}
//   pairs     one warp per particle, particles taken in cell order: the lanes
//             stream the 3^dim neighbour cells (contiguous runs along the last
//             axis) with coalesced loads, keep the tree points within h by
//             ballot, rank-sort them by (r^2, j), evaluate the pressure,
//             viscous, background-pressure and transport terms and the
//             density rate one pair per lane, and sum them in list order
//   corrector corrector, Shepard filter every 20 steps, boundary volume
//             fraction and bounce-back
//
// Layout (HBM, structure of arrays): position, velocity, transport velocity,
// force (+density rate in .w) and background force as 4-vectors of REAL;
// rho, old_rho, mass, nu as REAL arrays; neighbour lists [N][KCAP] (one list
// row is written by one warp, lane k writing entry k).
//
// The reference builds its kd-tree once per step, so in the force pass a
// moved particle is searched against start-of-step points and finds its own
// start-of-step point at distance |dt vt|; that self pair enters the Shepard
// filter and the boundary volume fraction.  The FP32 path takes that distance
// from the predictor displacement dt*vt, which FP32 positions cannot resolve.
// Densities read from neighbours in the corrector are their post-predictor
// values (old_rho), the order a parallel engine reads them in.
//
// FP32 storage.  The FP32 instantiation computes in float but stores a
// position as a float pair hi + lo (advanced by an error-free two-sum) and a
// density as its deviation from rho0 (rho, old_rho), with the float density
// rho0 + deviation in rfull for every reader other than the pressure
// P = P0 (rho/rho0 - 1) = P0 deviation/rho0.  Plain float storage decides the
// pressure term's sign switch (model.cpp:111-112) on rounding noise: after
// 1,000 steps of the 1,368-particle dam break its velocities are 2.8e-4 from
// FP64, these are 1.2e-6.  Box tests of boundary conditions read hi parts.
//
// Compiled with -fmad=false: the arithmetic rounds like the CPU oracle.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <vector>

#include "common.cuh"
#include "neighbors.cuh"
#include "sdpd.cuh"

namespace spg {

template <typename R> struct Vec4;
template <> struct Vec4<float> { using T = float4; };
template <> struct Vec4<double> { using T = double4; };

// float: compensated storage (hi + lo positions, density deviations)
template <typename R> constexpr bool kComp = sizeof(R) == 4;

template <typename R>
struct SdpdDev {
    int N, dim, step, stat;
    int self_step;   // self pair at |dt vt| (always in FP32)
    R h, dt, rho0, P0, alpha, g0, g1, g2;
    R acc2;      // largest r^2 with r^2 <= h^2 and sqrt(r^2) <= h (list predicate)
    double inv_cs;   // 1 / cell edge
    double rho0d;
    typename Vec4<R>::T *pos, *vel, *vt, *F, *Fbp, *pold;
    typename Vec4<R>::T *plo, *pold_lo;   // lo parts (float only)
    R *rho, *orho, *mass, *nu;
    R* rfull;    // float: rho0 + deviation; double: the densities themselves
    const uint8_t* fixed;
    // counting sort of the tree points by cell
    int *ccnt, *cstart;             // per cell: count (zero between steps), first sorted slot
    int* tcnt;                      // per tile of kScanTile cells: count, two buffers by step parity
    int ntile;
    int *ckey, *crank;              // per particle: cell, rank within the cell
    int* qkey;                      // per particle: cell of the moved position
    int* slot_of;                   // per particle: its slot in the cell order
    // cell-ordered copies (slot = cstart[cell] + rank), written by the scatter
    typename Vec4<R>::T *s_tp, *s_tplo;   // tree point (.w: particle index bits), lo part
    typename Vec4<R>::T *s_x, *s_xlo;     // current position (.w: mass), lo part
    typename Vec4<R>::T *s_v, *s_vt;      // velocity, transport velocity
    typename Vec4<R>::T* s_aux;           // {rho, P/rho^2, m/rho, nu}
    int *ncnt, *nidx;
    R *ndist, *ndw;
    R* ndij;     // D_ij per list entry, or nullptr when no species diffuse
    R *pr, *wv;  // per particle after the predictor: P/rho^2 and m/rho (read by pairs)
    int kcap;
    CellGrid g;
    int* flag;   // bit 1: list overflow, bit 2: NaN state
    // boundary conditions on v, nu, rho (boundarycondition.py:121-167)
    const int* type;
    int nbc;
    const double* bc_box;
    const int* bc_type;
    const int* bc_target;
    const double* bc_value;
};

// The boundary conditions that target v, nu or rho, in order: a particle
// inside the condition's box (and of its type) takes the value
// (applyBoundaryConditions, called after the predictor and after the
// corrector, simulate.cpp:88, 171).  Concentration targets are chem.cu's.
template <typename R, typename V>
__device__ __forceinline__ void flow_bcs(const SdpdDev<R>& D, int i, const V& p, V& v, R& rho) {
    // the density as the condition sees it; a stored deviation changes only
    // if the conditions leave a different density
    const double rin = kComp<R> ? D.rho0d + (double)rho : (double)rho;
    double rr = rin;
    for (int b = 0; b < D.nbc; b++) {
        const int tg = D.bc_target[b];
        if (tg >= SP_BC_C) continue;
        const double* bx = D.bc_box + 6 * b;
        const double px = (double)p.x, py = (double)p.y, pz = (double)p.z;
        if (!(px >= bx[0] && px <= bx[1] && py >= bx[2] && py <= bx[3] && pz >= bx[4] &&
              pz <= bx[5] && (D.bc_type[b] == 0 || D.bc_type[b] == D.type[i])))
            continue;
        const double* val = D.bc_value + 3 * b;
        if (tg == SP_BC_V) {
            v.x = (R)val[0];
            v.y = (R)val[1];
            v.z = (R)val[2];
        } else if (tg == SP_BC_NU) {
            D.nu[i] = (R)val[0];
        } else {
            rr = val[0];
        }
    }
    if (kComp<R>) {
        if (rr != rin) rho = (R)(rr - D.rho0d);
    } else {
        rho = (R)rr;
    }
}

// hi + lo += b, renormalised (two-sum, then fast two-sum)
__device__ __forceinline__ void comp_add(float& hi, float& lo, float b) {
    const float s = hi + b, bb = s - hi;
    const float e = (hi - (s - bb)) + (b - bb);
    const float l = lo + e, s2 = s + l;
    lo = l - (s2 - s);
    hi = s2;
}

constexpr int kScanThreads = 256;                 // cell scan: threads per CTA
constexpr int kScanTile = 4 * kScanThreads;       // cells per scan CTA (one int4 per thread)

// particle index carried in the .w of a cell-ordered tree point (bits only)
__device__ __forceinline__ float idx_bits(float, int j) { return __int_as_float(j); }
__device__ __forceinline__ double idx_bits(double, int j) {
    return __longlong_as_double((long long)j);
}
__device__ __forceinline__ int bits_idx(float w) { return __float_as_int(w); }
__device__ __forceinline__ int bits_idx(double w) { return (int)__double_as_longlong(w); }

// Cell of a coordinate, clamped to the grid.  Binning multiplies by 1/cs
// (cs = h (1 + 1e-7)): monotone in p and, with that margin, points within h
// of each other still fall in the same or adjacent cells.
template <typename R>
__device__ __forceinline__ int cellc(R p, const CellGrid& g, double inv_cs, int d) {
    if (d >= g.dim) return 0;
    int c = (int)floor(((double)p - g.lo[d]) * inv_cs);
    c = c < 0 ? 0 : c;
    return c >= g.nc[d] ? g.nc[d] - 1 : c;
}

template <typename V>
__device__ __forceinline__ int cell_key(const V& p, const CellGrid& g, double inv_cs) {
    return (cellc(p.x, g, inv_cs, 0) * g.nc[1] + cellc(p.y, g, inv_cs, 1)) * g.nc[2] +
           cellc(p.z, g, inv_cs, 2);
}

// take_step1 (simulate.cpp:56-109) + the cell key of the start-of-step point
template <typename R>
__global__ void sdpd_begin(SdpdDev<R> D) {
    using V = typename Vec4<R>::T;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= D.N) return;
    auto p = D.pos[i];
    V pl{};
    if (kComp<R>) pl = D.plo[i];
    auto v = D.vel[i];
    R rho = D.rho[i];
    if (isnan((double)p.x) || isinf((double)p.x) || isnan((double)p.y) || isinf((double)p.y) ||
        isnan((double)p.z) || isinf((double)p.z) || isnan((double)v.x) || isinf((double)v.x) ||
        isnan((double)v.y) || isinf((double)v.y) || isnan((double)v.z) || isinf((double)v.z) ||
        isnan((double)rho) || isinf((double)rho))
        atomicOr(D.flag, 2);
    // positions change only in the predictor, so the cell of this step's
    // start-of-step point is the cell of the last step's moved point
    const int c = D.step == 0 ? cell_key(p, D.g, D.inv_cs) : D.qkey[i];
    D.ckey[i] = c;
    D.crank[i] = atomicAdd(&D.ccnt[c], 1);
    {
        // the tile's count, one atomic per group of lanes on the same tile
        const int tile = c / kScanTile;
        const unsigned same = __match_any_sync(__activemask(), tile);
        if ((threadIdx.x & 31) == __ffs(same) - 1)
            atomicAdd(&D.tcnt[(D.step & 1) * D.ntile + tile], __popc(same));
    }
    int qc = c;
    D.pold[i] = p;
    if (kComp<R>) D.pold_lo[i] = pl;
    if (!D.stat && !D.fixed[i]) {
        const auto F = D.F[i];
        const auto Fb = D.Fbp[i];
        const R hdt = (R)0.5 * D.dt;
        v.x = v.x + hdt * F.x;
        v.y = v.y + hdt * F.y;
        v.z = v.z + hdt * F.z;
        auto t = v;
        t.x = v.x + hdt * Fb.x;
        t.y = v.y + hdt * Fb.y;
        t.z = v.z + hdt * Fb.z;
        if constexpr (kComp<R>) {
            comp_add(p.x, pl.x, D.dt * t.x);
            comp_add(p.y, pl.y, D.dt * t.y);
            comp_add(p.z, pl.z, D.dt * t.z);
            D.plo[i] = pl;
        } else {
            p.x = p.x + D.dt * t.x;
            p.y = p.y + D.dt * t.y;
            p.z = p.z + D.dt * t.z;
        }
        qc = cell_key(p, D.g, D.inv_cs);
        rho = rho + hdt * F.w;
        D.vel[i] = v;
        D.vt[i] = t;
        D.pos[i] = p;
        D.rho[i] = rho;
    }
    if (D.nbc) {
        flow_bcs(D, i, p, v, rho);
        D.vel[i] = v;
        D.rho[i] = rho;
    }
    auto F = D.F[i];
    F.x = D.g0; F.y = D.g1; F.z = D.g2; F.w = 0;
    D.F[i] = F;
    auto Fb = D.Fbp[i];
    Fb.x = 0; Fb.y = 0; Fb.z = 0; Fb.w = 0;
    D.Fbp[i] = Fb;
    D.orho[i] = rho;
    D.qkey[i] = qc;
    // the pressure term P/rho^2 and the volume m/rho of this particle, as the
    // force pass evaluates them for every pair it is in (model.cpp:105-120)
    if constexpr (kComp<R>) {
        const R rf = D.rho0 + rho;
        D.rfull[i] = rf;
        const R P = D.P0 * (rho / D.rho0);
        D.pr[i] = P / (rf * rf);
        D.wv[i] = D.mass[i] / rf;
    } else {
        const R P = D.P0 * (rho / D.rho0 - (R)1.0);
        D.pr[i] = P / (rho * rho);
        D.wv[i] = D.mass[i] / rho;
    }
}

// Exclusive scan of the per-cell counts into the cell starts (start[ncell_pad]
// = number of particles), resetting the counts to zero for the next step.
// One CTA per tile of kScanTile cells, with no waiting between CTAs: a tile's
// offset is the sum of the totals of the tiles before it, which sdpd_begin
// counted (buffer `par` = step parity); each CTA also zeroes its tile's count
// in the other buffer, the one the next step fills.  ncell_pad is a multiple
// of 16 and the padding cells stay empty.
__global__ void __launch_bounds__(kScanThreads) sdpd_cell_scan(int* cnt, int* start, int* tcnt,
                                                               int ntile, int par, int ncell_pad) {
    __shared__ int wsum[kScanThreads / 32];
    __shared__ int s_off;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int tile = blockIdx.x;
    const int* tc = tcnt + par * ntile;
    // the tiles before this one
    int before = 0;
    for (int t = tid; t < tile; t += kScanThreads) before += tc[t];
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) before += __shfl_xor_sync(SP_FULL, before, d);
    if (lane == 0) wsum[wid] = before;
    __syncthreads();
    if (tid == 0) {
        int o = 0;
        for (int w = 0; w < kScanThreads / 32; w++) o += wsum[w];
        s_off = o;
        tcnt[(1 - par) * ntile + tile] = 0;
    }
    __syncthreads();
    const int off = s_off;
    // this tile: 4 cells per thread as one int4 row
    const int c0 = tile * kScanTile + 4 * tid;
    int4 v = make_int4(0, 0, 0, 0);
    if (c0 < ncell_pad) v = reinterpret_cast<const int4*>(cnt)[c0 / 4];
    const int row = v.x + v.y + v.z + v.w;
    int incl = row;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(SP_FULL, incl, d);
        if (lane >= d) incl += t;
    }
    __syncthreads();   // wsum is reused
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    int wbefore = 0;
    for (int w = 0; w < wid; w++) wbefore += wsum[w];
    if (c0 < ncell_pad) {
        int run = off + wbefore + incl - row;
        int4 o;
        o.x = run; run += v.x;
        o.y = run; run += v.y;
        o.z = run; run += v.z;
        o.w = run;
        reinterpret_cast<int4*>(start)[c0 / 4] = o;
        reinterpret_cast<int4*>(cnt)[c0 / 4] = make_int4(0, 0, 0, 0);
    }
    if (tile == ntile - 1 && tid == kScanThreads - 1) {
        int tot = 0;
        for (int w = 0; w < kScanThreads / 32; w++) tot += wsum[w];
        start[ncell_pad] = off + tot;
    }
}

// Counting-sort scatter: particle i goes to slot cstart[cell] + rank, with
// the data the force pass and the corrector read about a neighbour packed
// into float4s (velocity .w: post-predictor density; transport velocity .w:
// 1 for a fixed particle).
template <typename R>
__global__ void sdpd_scatter(SdpdDev<R> D) {
    using V = typename Vec4<R>::T;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= D.N) return;
    const int sl = D.cstart[D.ckey[i]] + D.crank[i];
    D.slot_of[i] = sl;
    V tp = D.pold[i];
    tp.w = idx_bits((R)0, i);
    D.s_tp[sl] = tp;
    V x = D.pos[i];
    x.w = D.mass[i];
    D.s_x[sl] = x;
    if (kComp<R>) {
        D.s_tplo[sl] = D.pold_lo[i];
        D.s_xlo[sl] = D.plo[i];
    }
    V v = D.vel[i];
    v.w = D.orho[i];               // post-predictor density (Shepard filter)
    D.s_v[sl] = v;
    V t = D.vt[i];
    t.w = D.fixed[i] ? (R)1 : (R)0;
    D.s_vt[sl] = t;
    V a;
    a.x = D.rfull[i];
    a.y = D.pr[i];
    a.z = D.wv[i];
    a.w = D.nu[i];
    D.s_aux[sl] = a;
}

// Force pass of one step: find_neighbors against the step's tree points and
// pairwiseForce (particle.cpp:240-294, model.cpp:39-191), and with CORRECT
// the corrector take_step2 with filterDensity and the boundary volume
// fraction (simulate.cpp:132-173, model.cpp:194-329).
//
// One thread per particle, threads taking particles in cell order, so a
// warp's particles share neighbour cells and their cache lines.  The 3^dim
// cells around the query point are nine runs of consecutive slots in the
// cell-ordered copies; every tree point within h is insertion-sorted into the
// thread's list in shared memory by the key (r^2, j), the reference's list
// order.  The pairs are then evaluated in list order with the sums (forces,
// background force, density rate and the corrector's list sums) kept in
// registers, so the summation order is the reference's.  Every neighbour value
// comes from the cell-ordered copies, which nothing writes during the pass,
// so the corrector can run here: it writes only the particle's own state.
// Force pass of one step: find_neighbors against the step's tree points and
// pairwiseForce (particle.cpp:240-294, model.cpp:39-191), and with CORRECT
// the corrector take_step2 with filterDensity and the boundary volume
// fraction (simulate.cpp:132-173, model.cpp:194-329).
//
// One thread per particle, threads taking particles in cell order, so a
// warp's particles share neighbour cells and their cache lines.  The 3^dim
// cells around the query point are nine runs of consecutive slots in the
// cell-ordered copies; every tree point within h is insertion-sorted into the
// thread's list in shared memory by the key (r^2, j), the reference's list
// order.  The pairs are then evaluated in list order with the sums (forces,
// background force, density rate and the corrector's list sums) kept in
// registers, so the summation order is the reference's.  Every neighbour value
// comes from the cell-ordered copies, which nothing writes during the pass,
// so the corrector can run here: it writes only the particle's own state.
template <typename R> struct ListKey;
template <> struct ListKey<float> {   // r^2 >= 0 orders like its bit pattern
    using T = unsigned long long;
    __device__ static T make(float d2, int j) {
        return ((unsigned long long)__float_as_uint(d2) << 32) | (unsigned)j;
    }
    __device__ static float d2(T k) { return __uint_as_float((unsigned)(k >> 32)); }
    __device__ static int j(T k) { return (int)(unsigned)k; }
};
template <> struct ListKey<double> {
    using T = double2;   // (r^2, j as double)
    __device__ static T make(double d2, int j) { return make_double2(d2, (double)j); }
    __device__ static double d2(T k) { return k.x; }
    __device__ static int j(T k) { return (int)k.y; }
};
__device__ __forceinline__ bool key_less(unsigned long long a, unsigned long long b) { return a < b; }
__device__ __forceinline__ bool key_less(double2 a, double2 b) {
    return a.x < b.x || (a.x == b.x && a.y < b.y);
}

template <typename R> struct PairShape;
template <> struct PairShape<float> { static constexpr int TB = 64, MINB = 9; };
template <> struct PairShape<double> { static constexpr int TB = 64, MINB = 5; };

template <typename R, int KCAP, bool CORRECT>
__global__ void __launch_bounds__(PairShape<R>::TB, PairShape<R>::MINB)
    sdpd_pairs(SdpdDev<R> D, int first_step) {
    using V = typename Vec4<R>::T;
    using K = ListKey<R>;
    constexpr int TB = PairShape<R>::TB;
    // element k of thread t at [k * TB + t]: consecutive threads, consecutive banks
    __shared__ typename K::T list_all[KCAP * TB];
    typename K::T* list = list_all + threadIdx.x;
    const int s = blockIdx.x * TB + threadIdx.x;
    if (s >= D.N) return;
    const int i = bits_idx(D.s_tp[s].w);
    const int dim = D.dim;
    const R h = D.h;
    // at the first step of a run the lists come from the unmoved points (take_step1)
    const V q = first_step ? D.pold[i] : D.pos[i];
    V ql{};
    if (kComp<R>) ql = first_step ? D.pold_lo[i] : D.plo[i];
    const V ti = D.vt[i];
    R self_d2 = 0;
    if (D.self_step && !first_step) {
        const R a = D.dt * ti.x, b = D.dt * ti.y, c = D.dt * ti.z;
        self_d2 = a * a;
        if (dim > 1) self_d2 = self_d2 + b * b;
        if (dim > 2) self_d2 = self_d2 + c * c;
        if (D.stat || D.fixed[i]) self_d2 = 0;
    }
    const int key = first_step ? D.ckey[i] : D.qkey[i];
    const int n0 = D.g.nc[0], n1 = D.g.nc[1], n2 = D.g.nc[2];
    const int c2 = key % n2, c1 = (key / n2) % n1, c0 = key / (n2 * n1);
    const int zlo = c2 > 0 ? c2 - 1 : 0, zhi = c2 + 1 < n2 ? c2 + 1 : n2 - 1;
    const int kc = KCAP < D.kcap ? KCAP : D.kcap;
    const R acc2 = D.acc2;
    int m = 0;
    bool over = false;
    for (int a = c0 - 1; a <= c0 + 1; a++) {
        if (a < 0 || a >= n0) continue;
        for (int b = c1 - 1; b <= c1 + 1; b++) {
            if (b < 0 || b >= n1) continue;
            const int cb = (a * n1 + b) * n2;
            const int e = D.cstart[cb + zhi + 1];
            for (int sl = D.cstart[cb + zlo]; sl < e; sl++) {
                const V pt = D.s_tp[sl];
                const int j = bits_idx(pt.w);
                R e0 = q.x - pt.x, e1 = q.y - pt.y, e2 = q.z - pt.z;
                if constexpr (kComp<R>) {
                    const V pl = D.s_tplo[sl];
                    e0 = e0 + (ql.x - pl.x);
                    e1 = e1 + (ql.y - pl.y);
                    e2 = e2 + (ql.z - pl.z);
                }
                R d2 = 0;
                d2 = d2 + e0 * e0;
                if (dim > 1) d2 = d2 + e1 * e1;
                if (dim > 2) d2 = d2 + e2 * e2;
                if (D.self_step && j == i) d2 = self_d2;
                // d2 <= h^2 (kd_fix_rad_search.cpp:160-174) and sqrt(d2) <= h
                // (particle.cpp:160-162) in one compare: acc2 is the largest
                // value passing both (sqrt is correctly rounded and monotone)
                if (d2 > acc2 || d2 == (R)0) continue;
                if (m >= kc) {
                    over = true;
                    continue;
                }
                const typename K::T kk = K::make(d2, j);
                int k = m++;
                while (k > 0) {
                    const typename K::T prev = list[(k - 1) * TB];
                    if (!key_less(kk, prev)) break;
                    list[k * TB] = prev;
                    k--;
                }
                list[k * TB] = kk;
            }
        }
    }
    // pairs in list order
    const R alpha = D.alpha;
    const V xi = D.pos[i];
    V xli{};
    if (kComp<R>) xli = D.plo[i];
    const V vi = D.vel[i];
    const R rhoi = D.rfull[i], mi = D.mass[i], nui = D.nu[i], rho_i = D.rho[i];
    const R P0 = D.P0, rho0 = D.rho0;
    const R Pi = kComp<R> ? P0 * (rho_i / rho0) : P0 * (rhoi / rho0 - (R)1.0);
    const R pri = Pi / (rhoi * rhoi), npri = -Pi / (rhoi * rhoi), wi = D.wv[i];
    const R imi = (R)1.0 / mi;
    R Fx = D.g0, Fy = D.g1, Fz = D.g2, Bx = 0, By = 0, Bz = 0, Fr = 0;
    R num = 0, den = 0, vos = 0, vtot = 0, nw0 = 0, nw1 = 0, nw2 = 0;
    const size_t row = (size_t)i * D.kcap;
    for (int k = 0; k < m; k++) {
        const typename K::T kk = list[k * TB];
        const R d2 = K::d2(kk);
        const int j = K::j(kk);
        const int sl = D.slot_of[j];
        const R r = sqrt(d2);
        const R R_ = r / h;
        const R dWdr = alpha * ((R)-12 * r / (h * h)) * (((R)1 - R_) * ((R)1 - R_));
        D.nidx[row + k] = j;
        D.ndist[row + k] = r;
        D.ndw[row + k] = dWdr;
        const V xj = D.s_x[sl];      // .w: mass
        const V aux = D.s_aux[sl];   // rho, P/rho^2, m/rho, nu
        const R mj = xj.w, rhoj = aux.x;
        if (D.ndij) {
            // D_ij of add_to_neighbor_list (particle.cpp:181-187) from the
            // post-predictor densities, in the reference's operator order
            const R ih = (R)1.0 / h;
            const R ihsq = ih * ih;
            const R dhr = h - r;
            const R wfd = (R)-25.066903536973515383 * dhr * dhr * ihsq * ihsq * ihsq * ih;
            D.ndij[row + k] = (R)-2.0 * (mi * mj) / (mi + mj) * (rhoi + rhoj) / (rhoi * rhoj) *
                              d2 * wfd / (d2 + (R)0.01 * h * h);
        }
        if (R_ > (R)1.0 || r == (R)0) continue;
        const V vj4 = D.s_v[sl];     // .w: post-predictor density
        const V tj = D.s_vt[sl];     // .w: 1 when fixed
        R ex0 = xi.x - xj.x, ex1 = xi.y - xj.y, ex2 = xi.z - xj.z;
        if constexpr (kComp<R>) {
            const V xlj = D.s_xlo[sl];
            ex0 = ex0 + (xli.x - xlj.x);
            ex1 = ex1 + (xli.y - xlj.y);
            ex2 = ex2 + (xli.z - xlj.z);
        }
        R dx0 = 0, dx1 = 0, dx2 = 0, dv0 = 0, dv1 = 0, dv2 = 0, dvdx = 0;
        dx0 = ex0; dv0 = vi.x - vj4.x; dvdx = dvdx + dv0 * dx0;
        if (dim > 1) { dx1 = ex1; dv1 = vi.y - vj4.y; dvdx = dvdx + dv1 * dx1; }
        if (dim > 2) { dx2 = ex2; dv2 = vi.z - vj4.z; dvdx = dvdx + dv2 * dx2; }
        const R nuj = aux.w;
        const R prj = aux.y;                  // Pj / (rhoj * rhoj)
        R pg = pri + prj;
        if (pg < 0) pg = npri + prj;
        const R rh = r + (R)0.001 * h;
        const R fp = (R)-1.0 * mj * pg * dWdr / rh;
        const R fv = mj * ((R)2.0 * (nui * nuj) / (nui + nuj)) * ((R)1 / rh) * dWdr /
                     (rhoi * rhoj);
        const R wj = aux.z;                   // mj / rhoj
        const R ss = wi * wi + wj * wj;
        const R fbp = (R)-10.0 * P0 * imi * ss * dWdr / rh;
        const R a0 = ti.x - vi.x, a1 = ti.y - vi.y, a2 = ti.z - vi.z;
        const R b0 = tj.x - vj4.x, b1 = tj.y - vj4.y, b2 = tj.z - vj4.z;
        R ft[3];
        const R via[3] = {vi.x, vi.y, vi.z}, vja[3] = {vj4.x, vj4.y, vj4.z};
#pragma unroll
        for (int q2 = 0; q2 < 3; q2++) {
            const R T0 = (R)0.5 * ((rhoi * via[q2] * a0) + (rhoj * vja[q2] * b0));
            const R T1 = (R)0.5 * ((rhoi * via[q2] * a1) + (rhoj * vja[q2] * b1));
            const R T2 = (R)0.5 * ((rhoi * via[q2] * a2) + (rhoj * vja[q2] * b2));
            ft[q2] = imi * ss * (T0 * dx0 + T1 * dx1 + T2 * dx2) * dWdr / rh;
        }
        Fx = Fx + (fp * dx0 + fv * dv0 + ft[0]);
        Bx = Bx + fbp * dx0;
        if (dim > 1) { Fy = Fy + (fp * dx1 + fv * dv1 + ft[1]); By = By + fbp * dx1; }
        if (dim > 2) { Fz = Fz + (fp * dx2 + fv * dv2 + ft[2]); Bz = Bz + fbp * dx2; }
        const R tvi = (vi.x - ti.x) * dx0 + (vi.y - ti.y) * dx1 + (vi.z - ti.z) * dx2;
        const R tvj = (vj4.x - tj.x) * dx0 + (vj4.y - tj.y) * dx1 + (vj4.z - tj.z) * dx2;
        Fr = Fr + rhoi * wj * dvdx * ((R)1 / rh) * dWdr -
             wj * (rhoi * tvi + rhoj * tvj) * ((R)1.0 / rh) * dWdr;
        if constexpr (CORRECT) {
            // the list sums of filterDensity and of the boundary volume fraction
            const R omr = (R)1 - R_;
            const R W = alpha * (((R)1 + (R)3 * R_) * (omr * omr * omr));
            num = num + vj4.w * W;
            den = den + W;
            const R vv = wj * wj;
            const bool solid = tj.w != (R)0;
            if (solid) vos = vos + vv * W;
            vtot = vtot + vv * W;
            if (solid) {
                nw0 = nw0 + vv * dx0 * dWdr / rh;
                nw1 = nw1 + vv * dx1 * dWdr / rh;
                nw2 = nw2 + vv * dx2 * dWdr / rh;
            }
        }
    }
    D.ncnt[i] = m;
    if (over) atomicOr(D.flag, 1);
    V F;
    F.x = Fx; F.y = Fy; F.z = Fz; F.w = Fr;
    D.F[i] = F;
    V B;   // .w is zero since the predictor
    B.x = Bx; B.y = By; B.z = Bz; B.w = 0;
    D.Fbp[i] = B;
    if constexpr (CORRECT) {
        const bool fixed_i = D.fixed[i];
        const bool fluid = !fixed_i && !D.stat, wall = fixed_i && !D.stat;
        const R hdt = (R)0.5 * D.dt;
        V v = vi;
        R rho = rho_i;
        if (fluid) {
            v.x = v.x + hdt * F.x;
            v.y = v.y + hdt * F.y;
            v.z = v.z + hdt * F.z;
        }
        if ((fluid || wall) && D.step % 20 == 0) rho = num / den;
        if (fluid) {
            rho = rho + hdt * F.w;
            nw0 = nw0 / vtot;
            nw1 = nw1 / vtot;
            nw2 = nw2 / vtot;
            const R nn = sqrt(nw0 * nw0 + nw1 * nw1 + nw2 * nw2);
            const R n0 = -nw0 / nn, n1 = -nw1 / nn, n2n = -nw2 / nn;
            const R phi = fabs(vos / vtot);
            const R vdn = v.x * n0 + v.y * n1 + v.z * n2n;
            V t = ti;
            t.x = 0;
            if (dim > 1) t.y = 0;
            if (dim > 2) t.z = 0;
            D.vt[i] = t;
            if (phi >= (R)0.5) {   // applyBoundaryVolumeFraction, model.cpp:316-329
                const R mx = vdn > (R)0.0 ? vdn : (R)0.0;
                v.x = -v.x + (R)2.0 * mx * n0;
                if (dim > 1) v.y = -v.y + (R)2.0 * mx * n1;
                if (dim > 2) v.z = -v.z + (R)2.0 * mx * n2n;
            }
        }
        if (D.nbc) flow_bcs(D, i, xi, v, rho);   // applyBoundaryConditions, simulate.cpp:171
        D.vel[i] = v;
        D.rho[i] = rho;
        if (kComp<R>) D.rfull[i] = D.rho0 + rho;
    }
}

// take_step2 (simulate.cpp:132-173), filterDensity and the boundary volume
// fraction (model.cpp:194-329)
template <typename R>
__global__ void sdpd_corrector(SdpdDev<R> D) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= D.N) return;
    const bool fluid = !D.fixed[i] && !D.stat, wall = D.fixed[i] && !D.stat;
    const R h = D.h, alpha = D.alpha, hdt = (R)0.5 * D.dt;
    auto v = D.vel[i];
    const auto F = D.F[i];
    R rho = D.rho[i];
    const int m = D.ncnt[i];
    const size_t base = (size_t)i * D.kcap;
    if (fluid) {
        v.x = v.x + hdt * F.x;
        v.y = v.y + hdt * F.y;
        v.z = v.z + hdt * F.z;
    }
    if ((fluid || wall) && D.step % 20 == 0) {
        R num = 0, den = 0;
        for (int k = 0; k < m; k++) {
            const R r = D.ndist[base + k];
            const R R_ = r / h;
            if (R_ > (R)1.0 || r == (R)0) continue;
            const R omr = (R)1 - R_;
            const R W = alpha * (((R)1 + (R)3 * R_) * (omr * omr * omr));
            num = num + D.orho[D.nidx[base + k]] * W;
            den = den + W;
        }
        rho = num / den;
    }
    if (fluid) {
        rho = rho + hdt * F.w;
        const auto xi = D.pos[i];
        typename Vec4<R>::T xli{};
        if (kComp<R>) xli = D.plo[i];
        R nw0 = 0, nw1 = 0, nw2 = 0, vos = 0, vtot = 0;
        for (int k = 0; k < m; k++) {
            const R r = D.ndist[base + k];
            const R R_ = r / h;
            if (R_ > (R)1.0 || r == (R)0) continue;
            const int j = D.nidx[base + k];
            const R omr = (R)1 - R_;
            const R W = alpha * (((R)1 + (R)3 * R_) * (omr * omr * omr));
            const R dWdr = D.ndw[base + k];
            const auto xj = D.pos[j];
            R ex0 = xi.x - xj.x, ex1 = xi.y - xj.y, ex2 = xi.z - xj.z;
            if constexpr (kComp<R>) {
                const auto xlj = D.plo[j];
                ex0 = ex0 + (xli.x - xlj.x);
                ex1 = ex1 + (xli.y - xlj.y);
                ex2 = ex2 + (xli.z - xlj.z);
            }
            R dx0 = ex0, dx1 = 0, dx2 = 0;
            if (D.dim > 1) dx1 = ex1;
            if (D.dim > 2) dx2 = ex2;
            const R vj = D.mass[j] / (kComp<R> ? D.rho0 + D.orho[j] : D.orho[j]);
            const R vv = vj * vj;
            const bool solid = D.fixed[j];
            if (solid) vos = vos + vv * W;
            vtot = vtot + vv * W;
            if (solid) {
                const R rh = r + (R)0.001 * h;
                nw0 = nw0 + vv * dx0 * dWdr / rh;
                nw1 = nw1 + vv * dx1 * dWdr / rh;
                nw2 = nw2 + vv * dx2 * dWdr / rh;
            }
        }
        nw0 = nw0 / vtot;
        nw1 = nw1 / vtot;
        nw2 = nw2 / vtot;
        const R nn = sqrt(nw0 * nw0 + nw1 * nw1 + nw2 * nw2);
        const R n0 = -nw0 / nn, n1 = -nw1 / nn, n2 = -nw2 / nn;
        const R phi = fabs(vos / vtot);
        const R vdn = v.x * n0 + v.y * n1 + v.z * n2;
        auto t = D.vt[i];
        t.x = 0;
        if (D.dim > 1) t.y = 0;
        if (D.dim > 2) t.z = 0;
        D.vt[i] = t;
        if (phi >= (R)0.5) {                 // applyBoundaryVolumeFraction, model.cpp:316-329
            const R mx = vdn > (R)0.0 ? vdn : (R)0.0;
            v.x = -v.x + (R)2.0 * mx * n0;
            if (D.dim > 1) v.y = -v.y + (R)2.0 * mx * n1;
            if (D.dim > 2) v.z = -v.z + (R)2.0 * mx * n2;
        }
    }
    if (D.nbc) flow_bcs(D, i, D.pos[i], v, rho);   // applyBoundaryConditions, simulate.cpp:171
    D.vel[i] = v;
    D.rho[i] = rho;
    if (kComp<R>) D.rfull[i] = D.rho0 + rho;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct SdpdState {
    int prec = SP_PREC_F32;
    int N = 0, dim = 0, step = 0, kcap = 48, stat = 0, self_step = 1;
    double h = 0, dt = 0, rho0 = 0, P0 = 0, g[3] = {0, 0, 0};
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::vector<void*> allocs;
    void *pos = nullptr, *vel = nullptr, *vt = nullptr, *F = nullptr, *Fbp = nullptr,
         *pold = nullptr, *rho = nullptr, *orho = nullptr, *mass = nullptr,
         *nu = nullptr, *ndist = nullptr, *ndw = nullptr, *pr = nullptr, *wv = nullptr;
    // FP32 only: lo parts of positions (current, start of step) and the float
    // densities rho0 + deviation
    void *plo = nullptr, *pold_lo = nullptr, *rfull = nullptr;
    // cell-ordered copies (the lo parts in FP32 only)
    void *s_tp = nullptr, *s_tplo = nullptr, *s_x = nullptr, *s_xlo = nullptr, *s_v = nullptr,
         *s_vt = nullptr, *s_aux = nullptr;
    uint8_t* fixed = nullptr;
    int *ccnt = nullptr, *cstart = nullptr, *ckey = nullptr, *crank = nullptr, *qkey = nullptr,
        *slot_of = nullptr;
    int ncell_pad = 0;   // cells rounded up to a multiple of 16 (the scan's int4 rows)
    int ntile = 0;       // scan tiles of kScanTile cells
    int* tcnt = nullptr; // per tile counts, two buffers [2][ntile]
    int *ncnt = nullptr, *nidx = nullptr, *flag = nullptr;
    void* ndij = nullptr;
    // initial state (REAL-typed 4-vectors and densities) for sdpd_reset
    std::vector<unsigned char> init_pos, init_vel, init_rho, init_nu, init_lo, init_rfull;
    int* type = nullptr;
    int nbc = 0;
    double *bc_box = nullptr, *bc_value = nullptr;
    int *bc_type = nullptr, *bc_target = nullptr;
    CellGrid grid{};
    cudaGraphExec_t graph20 = nullptr;   // 20 steps starting at a multiple of 20 (>= 20)
};

static bool sd_alloc(SdpdState* s, void** p, size_t bytes, std::string* err) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *err = std::string("cudaMalloc (SDPD state): ") + cudaGetErrorString(e);
        return false;
    }
    s->allocs.push_back(*p);
    return true;
}

template <typename R>
static SdpdDev<R> dev_view(SdpdState* s) {
    using V = typename Vec4<R>::T;
    SdpdDev<R> D{};
    D.N = s->N;
    D.dim = s->dim;
    D.step = s->step;
    D.stat = s->stat;
    D.self_step = s->self_step;
    D.h = (R)s->h;
    D.dt = (R)s->dt;
    D.rho0 = (R)s->rho0;
    D.rho0d = s->rho0;
    D.P0 = (R)s->P0;
    const R h = (R)s->h;
    D.alpha = s->dim == 3 ? (R)105 / ((R)16 * (R)M_PI * h * h * h)
            : s->dim == 2 ? (R)5 / ((R)M_PI * h * h) : h;
    // the list predicate d2 <= h*h && sqrt(d2) <= h as one compare: sqrt is
    // correctly rounded and monotone here and on the device, so the largest
    // passing value is found by stepping down from h*h
    {
        R a2 = h * h;
        while (a2 > (R)0 && std::sqrt(a2) > h) a2 = std::nextafter(a2, (R)0);
        D.acc2 = a2;
    }
    D.g0 = (R)s->g[0];
    D.g1 = (R)s->g[1];
    D.g2 = (R)s->g[2];
    D.pos = (V*)s->pos; D.vel = (V*)s->vel; D.vt = (V*)s->vt; D.F = (V*)s->F; D.Fbp = (V*)s->Fbp;
    D.pold = (V*)s->pold;
    D.plo = (V*)s->plo; D.pold_lo = (V*)s->pold_lo;
    D.rho = (R*)s->rho; D.orho = (R*)s->orho; D.mass = (R*)s->mass; D.nu = (R*)s->nu;
    D.rfull = kComp<R> ? (R*)s->rfull : (R*)s->rho;
    D.fixed = s->fixed;
    D.ccnt = s->ccnt; D.cstart = s->cstart; D.ckey = s->ckey; D.crank = s->crank;
    D.tcnt = s->tcnt; D.ntile = s->ntile;
    D.qkey = s->qkey;
    D.slot_of = s->slot_of;
    D.s_tp = (V*)s->s_tp; D.s_tplo = (V*)s->s_tplo; D.s_x = (V*)s->s_x; D.s_xlo = (V*)s->s_xlo;
    D.s_v = (V*)s->s_v; D.s_vt = (V*)s->s_vt; D.s_aux = (V*)s->s_aux;
    D.ncnt = s->ncnt; D.nidx = s->nidx; D.ndist = (R*)s->ndist; D.ndw = (R*)s->ndw;
    D.ndij = (R*)s->ndij;
    D.pr = (R*)s->pr;
    D.wv = (R*)s->wv;
    D.type = s->type;
    D.nbc = s->nbc;
    D.bc_box = s->bc_box;
    D.bc_type = s->bc_type;
    D.bc_target = s->bc_target;
    D.bc_value = s->bc_value;
    D.kcap = s->kcap;
    D.g = s->grid;
    D.inv_cs = 1.0 / s->grid.cs;
    D.flag = s->flag;
    return D;
}

template <typename R>
static bool upload(SdpdState* s, const sp_scenario& sc, std::string* err) {
    using V = typename Vec4<R>::T;
    const int N = sc.num_particles;
    const size_t v4 = sizeof(V) * N, r1 = sizeof(R) * N;
    void** four[] = {&s->pos, &s->vel, &s->vt, &s->F, &s->Fbp, &s->pold,
                     &s->s_tp, &s->s_x, &s->s_v, &s->s_vt, &s->s_aux};
    for (void** p : four)
        if (!sd_alloc(s, p, v4, err)) return false;
    void** ones[] = {&s->rho, &s->orho, &s->mass, &s->nu, &s->pr, &s->wv};
    for (void** p : ones)
        if (!sd_alloc(s, p, r1, err)) return false;
    if (kComp<R>) {
        void** lo[] = {&s->plo, &s->pold_lo, &s->s_tplo, &s->s_xlo};
        for (void** p : lo)
            if (!sd_alloc(s, p, v4, err)) return false;
        if (!sd_alloc(s, &s->rfull, r1, err)) return false;
    }
    std::vector<V> pos(N), zero(N), vel(N), lo(N);
    std::vector<R> rho(N), mass(N), nu(N), rf(N);
    for (int i = 0; i < N; i++) {
        pos[i].x = (R)sc.x[3 * i]; pos[i].y = (R)sc.x[3 * i + 1]; pos[i].z = (R)sc.x[3 * i + 2];
        pos[i].w = 0;
        zero[i].x = zero[i].y = zero[i].z = zero[i].w = 0;
        vel[i] = zero[i];
        lo[i] = zero[i];
        if (sc.v) { vel[i].x = (R)sc.v[3 * i]; vel[i].y = (R)sc.v[3 * i + 1]; vel[i].z = (R)sc.v[3 * i + 2]; }
        rho[i] = (R)sc.rho[i];
        if (kComp<R>) {
            lo[i].x = (R)(sc.x[3 * i] - (double)pos[i].x);
            lo[i].y = (R)(sc.x[3 * i + 1] - (double)pos[i].y);
            lo[i].z = (R)(sc.x[3 * i + 2] - (double)pos[i].z);
            rho[i] = (R)(sc.rho[i] - sc.rho0);
            rf[i] = (R)sc.rho0 + rho[i];
        }
        mass[i] = (R)sc.mass[i];
        nu[i] = (R)sc.nu[i];
    }
    s->init_pos.assign((unsigned char*)pos.data(), (unsigned char*)pos.data() + v4);
    s->init_vel.assign((unsigned char*)vel.data(), (unsigned char*)vel.data() + v4);
    s->init_rho.assign((unsigned char*)rho.data(), (unsigned char*)rho.data() + r1);
    s->init_nu.assign((unsigned char*)nu.data(), (unsigned char*)nu.data() + r1);
    if (kComp<R>) {
        s->init_lo.assign((unsigned char*)lo.data(), (unsigned char*)lo.data() + v4);
        s->init_rfull.assign((unsigned char*)rf.data(), (unsigned char*)rf.data() + r1);
        cudaMemcpyAsync(s->plo, lo.data(), v4, cudaMemcpyHostToDevice, s->st);
        cudaMemcpyAsync(s->rfull, rf.data(), r1, cudaMemcpyHostToDevice, s->st);
    }
    // F, Fbp, vt start at zero: the engine reads them before first writing
    // them (particle.cpp:70-83), the oracle zero-initialises them
    cudaMemcpyAsync(s->pos, pos.data(), v4, cudaMemcpyHostToDevice, s->st);
    cudaMemcpyAsync(s->vel, vel.data(), v4, cudaMemcpyHostToDevice, s->st);
    cudaMemcpyAsync(s->vt, zero.data(), v4, cudaMemcpyHostToDevice, s->st);
    cudaMemcpyAsync(s->F, zero.data(), v4, cudaMemcpyHostToDevice, s->st);
    cudaMemcpyAsync(s->Fbp, zero.data(), v4, cudaMemcpyHostToDevice, s->st);
    cudaMemcpyAsync(s->rho, rho.data(), r1, cudaMemcpyHostToDevice, s->st);
    cudaMemcpyAsync(s->orho, rho.data(), r1, cudaMemcpyHostToDevice, s->st);
    cudaMemcpyAsync(s->mass, mass.data(), r1, cudaMemcpyHostToDevice, s->st);
    cudaMemcpyAsync(s->nu, nu.data(), r1, cudaMemcpyHostToDevice, s->st);
    if (!sd_alloc(s, &s->ndist, sizeof(R) * (size_t)N * s->kcap, err)) return false;
    if (!sd_alloc(s, &s->ndw, sizeof(R) * (size_t)N * s->kcap, err)) return false;
    cudaError_t e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) {
        *err = std::string("SDPD upload: ") + cudaGetErrorString(e);
        return false;
    }
    return true;
}

SdpdState* sdpd_create(const sp_scenario& sc, int precision, int self_step, cudaStream_t st,
                       std::string* err) {
    SdpdState* s = new SdpdState();
    s->prec = precision == SP_PREC_F64 ? SP_PREC_F64 : SP_PREC_F32;
    s->self_step = s->prec == SP_PREC_F32 || self_step ? 1 : 0;
    s->N = sc.num_particles;
    s->dim = sc.dimension;
    s->h = sc.h;
    s->dt = sc.dt;
    s->rho0 = sc.rho0;
    s->P0 = sc.P0;
    s->stat = sc.static_domain ? 1 : 0;
    for (int d = 0; d < 3; d++) s->g[d] = sc.gravity[d];
    s->st = st;
    cudaEventCreate(&s->e0);
    cudaEventCreate(&s->e1);
    // cell grid over the initial bounding box grown by 4h on every side;
    // particles outside it fall into the edge cells (still exact, slower)
    s->grid = make_grid(sc.x, s->N, s->dim, sc.h);
    for (int d = 0; d < s->dim; d++) {
        s->grid.lo[d] -= 4 * s->grid.cs;
        s->grid.nc[d] += 8;
    }
    s->grid.ncell = s->grid.nc[0] * s->grid.nc[1] * s->grid.nc[2];
    s->ncell_pad = (s->grid.ncell + 15) / 16 * 16;
    s->ntile = (s->ncell_pad + kScanTile - 1) / kScanTile;
    const int N = s->N;
    bool ok = sd_alloc(s, (void**)&s->fixed, N, err) &&
              sd_alloc(s, (void**)&s->type, sizeof(int) * N, err) &&
              sd_alloc(s, (void**)&s->ccnt, sizeof(int) * s->ncell_pad, err) &&
              sd_alloc(s, (void**)&s->cstart, sizeof(int) * (s->ncell_pad + 4), err) &&
              sd_alloc(s, (void**)&s->tcnt, sizeof(int) * 2 * s->ntile, err) &&
              sd_alloc(s, (void**)&s->ckey, sizeof(int) * N, err) &&
              sd_alloc(s, (void**)&s->crank, sizeof(int) * N, err) &&
              sd_alloc(s, (void**)&s->qkey, sizeof(int) * N, err) &&
              sd_alloc(s, (void**)&s->slot_of, sizeof(int) * N, err) &&
              sd_alloc(s, (void**)&s->ncnt, sizeof(int) * N, err) &&
              sd_alloc(s, (void**)&s->nidx, sizeof(int) * (size_t)N * s->kcap, err) &&
              sd_alloc(s, (void**)&s->flag, sizeof(int), err);
    if (ok && sc.num_bcs > 0) {
        const int nb = sc.num_bcs;
        s->nbc = nb;
        ok = sd_alloc(s, (void**)&s->bc_box, sizeof(double) * 6 * nb, err) &&
             sd_alloc(s, (void**)&s->bc_value, sizeof(double) * 3 * nb, err) &&
             sd_alloc(s, (void**)&s->bc_type, sizeof(int) * nb, err) &&
             sd_alloc(s, (void**)&s->bc_target, sizeof(int) * nb, err);
        if (ok) {
            cudaMemcpyAsync(s->bc_box, sc.bc_box, sizeof(double) * 6 * nb, cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(s->bc_value, sc.bc_value, sizeof(double) * 3 * nb, cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(s->bc_type, sc.bc_type, sizeof(int) * nb, cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(s->bc_target, sc.bc_target, sizeof(int) * nb, cudaMemcpyHostToDevice, st);
        }
    }
    if (ok) {
        cudaMemcpyAsync(s->type, sc.type, sizeof(int) * N, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(s->fixed, sc.fixed, N, cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(s->ncnt, 0, sizeof(int) * N, st);
        cudaMemsetAsync(s->ccnt, 0, sizeof(int) * s->ncell_pad, st);   // the scan keeps it zero
        cudaMemsetAsync(s->tcnt, 0, sizeof(int) * 2 * s->ntile, st);
        ok = s->prec == SP_PREC_F64 ? upload<double>(s, sc, err) : upload<float>(s, sc, err);
    }
    if (!ok) {
        sdpd_destroy(s);
        return nullptr;
    }
    return s;
}

void sdpd_destroy(SdpdState* s) {
    if (!s) return;
    if (s->graph20) cudaGraphExecDestroy(s->graph20);
    for (void* p : s->allocs) cudaFree(p);
    if (s->e0) cudaEventDestroy(s->e0);
    if (s->e1) cudaEventDestroy(s->e1);
    delete s;
}

// one part of a step: 0 predictor (begin); 1 lists + forces (scan, scatter,
// pairs), with the corrector fused into the pairs when `correct`; 2 the
// corrector on its own (for callers that read the force-pass state in between)
template <typename R>
static void enqueue_part(SdpdState* s, int step, int part, bool correct) {
    const int N = s->N, tb = 128, nb = (N + tb - 1) / tb;
    SdpdDev<R> D = dev_view<R>(s);
    D.step = step;
    if (part == 0) {
        sdpd_begin<R><<<nb, tb, 0, s->st>>>(D);
    } else if (part == 1) {
        sdpd_cell_scan<<<s->ntile, kScanThreads, 0, s->st>>>(s->ccnt, s->cstart, s->tcnt,
                                                             s->ntile, step & 1, s->ncell_pad);
        sdpd_scatter<R><<<nb, tb, 0, s->st>>>(D);
        constexpr int TB = PairShape<R>::TB;
        const int grid = (N + TB - 1) / TB;
        if (correct)
            sdpd_pairs<R, 48, true><<<grid, TB, 0, s->st>>>(D, step == 0);
        else
            sdpd_pairs<R, 48, false><<<grid, TB, 0, s->st>>>(D, step == 0);
    } else {
        sdpd_corrector<R><<<nb, tb, 0, s->st>>>(D);
    }
}

// one step: begin, scan, scatter, pairs + corrector (kSdpdLaunchesPerStep)
template <typename R>
static void enqueue_step(SdpdState* s, int step) {
    enqueue_part<R>(s, step, 0, true);
    enqueue_part<R>(s, step, 1, true);
}

template <typename R>
static int advance_t(SdpdState* s, int nsteps, double* ms, long long* launches, std::string* err) {
    cudaMemsetAsync(s->flag, 0, sizeof(int), s->st);
    cudaEventRecord(s->e0, s->st);
    long long l = 0;
    int k = 0;
    while (k < nsteps) {
        if (s->step >= 20 && s->step % 20 == 0 && nsteps - k >= 20) {
            // steps only differ through step % 20 (Shepard filter) and the
            // first step, so one captured block of 20 replays anywhere >= 20
            if (!s->graph20) {
                cudaGraph_t g;
                cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal);
                for (int q = 0; q < 20; q++) enqueue_step<R>(s, 20 + q);
                cudaError_t e = cudaStreamEndCapture(s->st, &g);
                if (e == cudaSuccess) e = cudaGraphInstantiate(&s->graph20, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) {
                    *err = std::string("SDPD graph capture: ") + cudaGetErrorString(e);
                    return SP_E_CUDA;
                }
            }
            cudaGraphLaunch(s->graph20, s->st);
            l += 20 * kSdpdLaunchesPerStep;
            k += 20;
            s->step += 20;
        } else {
            enqueue_step<R>(s, s->step);
            l += kSdpdLaunchesPerStep;
            k++;
            s->step++;
        }
    }
    cudaEventRecord(s->e1, s->st);
    int flag = 0;
    cudaMemcpyAsync(&flag, s->flag, sizeof(int), cudaMemcpyDeviceToHost, s->st);
    cudaError_t e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) {
        *err = std::string("SDPD step: ") + cudaGetErrorString(e);
        return SP_E_CUDA;
    }
    float t = 0;
    cudaEventElapsedTime(&t, s->e0, s->e1);
    *ms = t;
    *launches = l;
    if (flag & 1) {
        *err = "SDPD: a particle has more neighbours than the list capacity (48)";
        return SP_E_UNSUPPORTED;
    }
    if (flag & 2) {
        *err = "SDPD: NaN/inf in particle state (particle.cpp:88-126)";
        return SP_E_TRAJECTORY;
    }
    return SP_OK;
}

int sdpd_advance(SdpdState* s, int nsteps, double* ms, long long* launches, std::string* err) {
    return s->prec == SP_PREC_F64 ? advance_t<double>(s, nsteps, ms, launches, err)
                                  : advance_t<float>(s, nsteps, ms, launches, err);
}

template <typename R>
static int get_state_t(SdpdState* s, double* x, double* v, double* rho, std::string* err) {
    using V = typename Vec4<R>::T;
    const int N = s->N;
    std::vector<V> p(N), u(N), pl(N);
    std::vector<R> r(N);
    cudaMemcpy(p.data(), s->pos, sizeof(V) * N, cudaMemcpyDeviceToHost);
    if (kComp<R>) cudaMemcpy(pl.data(), s->plo, sizeof(V) * N, cudaMemcpyDeviceToHost);
    cudaMemcpy(u.data(), s->vel, sizeof(V) * N, cudaMemcpyDeviceToHost);
    cudaError_t e = cudaMemcpy(r.data(), kComp<R> ? s->rfull : s->rho, sizeof(R) * N,
                               cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        *err = std::string("SDPD state copy: ") + cudaGetErrorString(e);
        return SP_E_CUDA;
    }
    for (int i = 0; i < N; i++) {
        if (x) { x[3 * i] = p[i].x; x[3 * i + 1] = p[i].y; x[3 * i + 2] = p[i].z; }
        if (x && kComp<R>) {
            x[3 * i] += (double)pl[i].x;
            x[3 * i + 1] += (double)pl[i].y;
            x[3 * i + 2] += (double)pl[i].z;
        }
        if (v) { v[3 * i] = u[i].x; v[3 * i + 1] = u[i].y; v[3 * i + 2] = u[i].z; }
        if (rho) rho[i] = r[i];
    }
    return SP_OK;
}

int sdpd_get_state(SdpdState* s, double* x, double* v, double* rho, std::string* err) {
    return s->prec == SP_PREC_F64 ? get_state_t<double>(s, x, v, rho, err)
                                  : get_state_t<float>(s, x, v, rho, err);
}

template <typename R>
static int copy_nbr_t(SdpdState* s, int kmax, int* count, int* idx, double* dist, double* dwdr,
                      std::string* err) {
    const int N = s->N, K = s->kcap;
    std::vector<int> c(N), ix((size_t)N * K);
    std::vector<R> d((size_t)N * K), w((size_t)N * K);
    cudaMemcpy(c.data(), s->ncnt, sizeof(int) * N, cudaMemcpyDeviceToHost);
    cudaMemcpy(ix.data(), s->nidx, sizeof(int) * ix.size(), cudaMemcpyDeviceToHost);
    cudaMemcpy(d.data(), s->ndist, sizeof(R) * d.size(), cudaMemcpyDeviceToHost);
    cudaError_t e = cudaMemcpy(w.data(), s->ndw, sizeof(R) * w.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        *err = std::string("SDPD list copy: ") + cudaGetErrorString(e);
        return SP_E_CUDA;
    }
    for (int i = 0; i < N; i++) {
        if (c[i] > kmax) {
            *err = "kmax smaller than a neighbour count";
            return SP_E_INVALID;
        }
        count[i] = c[i];
        for (int k = 0; k < c[i]; k++) {
            idx[(size_t)i * kmax + k] = ix[(size_t)i * K + k];
            if (dist) dist[(size_t)i * kmax + k] = d[(size_t)i * K + k];
            if (dwdr) dwdr[(size_t)i * kmax + k] = w[(size_t)i * K + k];
        }
    }
    return SP_OK;
}

int sdpd_copy_neighbors(SdpdState* s, int kmax, int* count, int* idx, double* dist, double* dwdr,
                        double* dij, std::string* err) {
    (void)dij;
    return s->prec == SP_PREC_F64 ? copy_nbr_t<double>(s, kmax, count, idx, dist, dwdr, err)
                                  : copy_nbr_t<float>(s, kmax, count, idx, dist, dwdr, err);
}

// ---------------------------------------------------------------------------
// coupling with the NSM (moving domain with species)
// ---------------------------------------------------------------------------
int sdpd_enable_dij(SdpdState* s, std::string* err) {
    if (s->ndij) return SP_OK;
    const size_t rb = s->prec == SP_PREC_F64 ? sizeof(double) : sizeof(float);
    if (!sd_alloc(s, &s->ndij, rb * (size_t)s->N * s->kcap, err)) return SP_E_NOMEM;
    return SP_OK;
}

int sdpd_reset(SdpdState* s, std::string* err) {
    const size_t v4 = s->init_pos.size(), r1 = s->init_rho.size();
    cudaMemcpyAsync(s->pos, s->init_pos.data(), v4, cudaMemcpyHostToDevice, s->st);
    cudaMemcpyAsync(s->vel, s->init_vel.data(), v4, cudaMemcpyHostToDevice, s->st);
    cudaMemsetAsync(s->vt, 0, v4, s->st);
    cudaMemsetAsync(s->F, 0, v4, s->st);
    cudaMemsetAsync(s->Fbp, 0, v4, s->st);
    cudaMemcpyAsync(s->rho, s->init_rho.data(), r1, cudaMemcpyHostToDevice, s->st);
    cudaMemcpyAsync(s->orho, s->init_rho.data(), r1, cudaMemcpyHostToDevice, s->st);
    cudaMemcpyAsync(s->nu, s->init_nu.data(), r1, cudaMemcpyHostToDevice, s->st);
    if (s->plo) cudaMemcpyAsync(s->plo, s->init_lo.data(), v4, cudaMemcpyHostToDevice, s->st);
    if (s->rfull)
        cudaMemcpyAsync(s->rfull, s->init_rfull.data(), r1, cudaMemcpyHostToDevice, s->st);
    cudaMemsetAsync(s->ncnt, 0, sizeof(int) * s->N, s->st);
    cudaMemsetAsync(s->ccnt, 0, sizeof(int) * s->ncell_pad, s->st);
    cudaMemsetAsync(s->tcnt, 0, sizeof(int) * 2 * s->ntile, s->st);
    cudaMemsetAsync(s->flag, 0, sizeof(int), s->st);
    cudaError_t e = cudaStreamSynchronize(s->st);   // host staging buffers stay valid
    if (e != cudaSuccess) {
        *err = std::string("SDPD reset: ") + cudaGetErrorString(e);
        return SP_E_CUDA;
    }
    s->step = 0;
    return SP_OK;
}

void sdpd_enqueue_step(SdpdState* s) {
    if (s->prec == SP_PREC_F64) enqueue_step<double>(s, s->step);
    else enqueue_step<float>(s, s->step);
    s->step++;
}

template <typename R>
static void enqueue_phase_t(SdpdState* s, int phase) {
    enqueue_part<R>(s, s->step, phase, false);
    if (phase == 2) s->step++;
}

void sdpd_enqueue_phase(SdpdState* s, int phase) {
    if (s->prec == SP_PREC_F64) enqueue_phase_t<double>(s, phase);
    else enqueue_phase_t<float>(s, phase);
}

SdpdLists sdpd_lists(SdpdState* s) {
    SdpdLists L;
    L.count = s->ncnt;
    L.idx = s->nidx;
    L.dij = s->ndij;
    L.rho = s->prec == SP_PREC_F64 ? s->rho : s->rfull;   // full densities
    L.dist = s->ndist;
    L.dwdr = s->ndw;
    L.mass = s->mass;
    L.pos = s->pos;
    L.kcap = s->kcap;
    L.f64 = s->prec == SP_PREC_F64;
    L.step = s->step;
    return L;
}

template <typename R>
__global__ void sdpd_volumes(int n, const double* mass, const R* rho, float* vol, float* ivol) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double r = (double)rho[i];
    vol[i] = (float)(mass[i] / r);     // simulate_rdme.cpp:123, 247
    ivol[i] = (float)(r / mass[i]);
}

void sdpd_launch_volumes(SdpdState* s, const double* mass, float* vol, float* ivol) {
    const int n = s->N, tb = 256;
    if (s->prec == SP_PREC_F64)
        sdpd_volumes<double><<<(n + tb - 1) / tb, tb, 0, s->st>>>(n, mass, (const double*)s->rho, vol, ivol);
    else
        sdpd_volumes<float><<<(n + tb - 1) / tb, tb, 0, s->st>>>(n, mass, (const float*)s->rfull, vol, ivol);
}

template <typename R>
__global__ void sdpd_state_out(SdpdDev<R> D, double* x, double* v, double* rho) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= D.N) return;
    const auto p = D.pos[i];
    const auto u = D.vel[i];
    if (x) { x[3 * i] = p.x; x[3 * i + 1] = p.y; x[3 * i + 2] = p.z; }
    if (x && kComp<R>) {
        const auto pl = D.plo[i];
        x[3 * i] = (double)p.x + (double)pl.x;
        x[3 * i + 1] = (double)p.y + (double)pl.y;
        x[3 * i + 2] = (double)p.z + (double)pl.z;
    }
    if (v) { v[3 * i] = u.x; v[3 * i + 1] = u.y; v[3 * i + 2] = u.z; }
    if (rho) rho[i] = D.rfull[i];
}

void sdpd_launch_state_out(SdpdState* s, double* x, double* v, double* rho) {
    const int n = s->N, tb = 256;
    if (s->prec == SP_PREC_F64)
        sdpd_state_out<double><<<(n + tb - 1) / tb, tb, 0, s->st>>>(dev_view<double>(s), x, v, rho);
    else
        sdpd_state_out<float><<<(n + tb - 1) / tb, tb, 0, s->st>>>(dev_view<float>(s), x, v, rho);
}

int sdpd_check_flag(SdpdState* s, std::string* err) {
    int flag = 0;
    cudaMemcpyAsync(&flag, s->flag, sizeof(int), cudaMemcpyDeviceToHost, s->st);
    cudaError_t e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) {
        *err = std::string("SDPD step: ") + cudaGetErrorString(e);
        return SP_E_CUDA;
    }
    if (flag & 1) {
        *err = "SDPD: a particle has more neighbours than the list capacity (48)";
        return SP_E_UNSUPPORTED;
    }
    if (flag & 2) {
        *err = "SDPD: NaN/inf in particle state (particle.cpp:88-126)";
        return SP_E_TRAJECTORY;
    }
    return SP_OK;
}

}  // namespace spg
