// fno.cu — the surrogate network (a FiLM-conditioned Fourier neural operator)
// run and trained by hand-written kernels: forward, backward and Adam.
//
// Network and parameter layout: include/spgpu.h (sp_fno_*).  Fields are
// [batch][channel][n*n] fp32; weights are read as bf16 (a copy refreshed by
// the Adam kernel) and every product is accumulated in fp32.
//
// Work per sample is small and the contractions are width-32 channel mixes
// (2 x 32 x 32 flops per voxel and layer against 256 bytes of field traffic,
// 8 flop/byte), so the kernels are bound by memory and launch latency.  The
// channel mixes, the truncated DFTs and the per-mode complex mixes run on
// the tensor cores as mma.sync bf16, the channel mixes' weight gradients as
// mma.sync TF32, with fp32 operands split into a high part and the rounding
// of the remainder so that the sums keep fp32-level accuracy; shapes outside
// the tiles keep the fp32 CUDA-core kernels.  A training step (about 70 launches) is captured once per
// batch size as a CUDA graph and replayed.
//
// Kernels:
//   fno_pointwise    channel mix at every voxel (lift, the layers' linear
//                    paths, the projection, and their transposes in the
//                    backward pass), with fused bias, spectral addend, FiLM,
//                    GELU and GELU' epilogues; fno_pointwise_tc on the
//                    tensor cores where cout is a multiple of 16
//   fno_analysis     truncated 2-D DFT of each channel plane (rfft2 on the
//                    kept modes), scaled per ky; fno_analysis_tc on the
//                    tensor cores where n % 16 == 0 and 2m <= 32
//   fno_synthesis    its adjoint / the truncated inverse real DFT (and
//                    fno_synthesis_tc)
//   fno_mix          per-mode complex channel mixing (forward, and the
//                    conjugate transpose for the backward pass);
//                    fno_mix_tc on the tensor cores for width 16, 32, 64
//   fno_mix_wgrad    per-mode weight gradient, a reduction over the batch
//                    (fno_mix_wgrad_tc for width 16, 32)
//   fno_wgrad_*      pointwise weight gradients: per-tile partial products
//                    on the tensor cores, then an ordered reduction
//                    (deterministic)
//   fno_film_back    GELU' and the FiLM scale/shift gradients per plane
//   fno_dense*       the conditioning MLP and its gradients
//   fno_mse*         loss and output gradient
//   fno_adam         Adam step on the fp32 parameters, bf16 copy refresh
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/spgpu.h"

namespace spg {
namespace fno {

constexpr int kTile = 128;      // voxels per CTA in the pointwise weight-gradient pass
constexpr int kLossBlocks = 512;

__device__ __forceinline__ float bfv(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }

// fp32 -> bf16, round to nearest even (NaN kept quiet)
__host__ __device__ inline uint16_t to_bf16(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

// GELU (erf form) and its derivative
__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float x) {
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) +
           x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// ---------------------------------------------------------------------------
// pointwise channel mix
// ---------------------------------------------------------------------------
struct PW {
    const float* in;
    long long in_bs;       // batch stride of `in` in floats (0: one input for the batch)
    int cin, cout, P, B;
    const uint16_t* w;     // trans = 0: W[o*cin + i]; trans = 1: W[i*cout + o]
    int trans;
    const uint16_t* bias;  // [cout] or null
    const float* add;      // [B][cout][P] or null
    const float* film;     // g0 = film[b*fs + o], g1 = film[b*fs + cout + o]; null = none
    int fs;
    int act;               // 0 none, 1 GELU, 2 multiply by GELU'(gate)
    const float* gate;     // [B][cout][P] for act 2
    float* pre;            // null or [B][cout][P]: the value before FiLM and activation
    float* out;            // [B][cout][P]
    int accumulate;        // out += result
};

template <int CO>
__global__ void __launch_bounds__(128) fno_pointwise(PW a) {
    extern __shared__ float ws[];          // [cin][cout] weights, then [cout] bias
    const int nw = a.cin * a.cout;
    for (int e = threadIdx.x; e < nw; e += blockDim.x) {
        int i, o;
        if (a.trans) { i = e / a.cout; o = e % a.cout; }
        else         { o = e / a.cin;  i = e % a.cin; }
        ws[i * a.cout + o] = bfv(a.w[e]);
    }
    for (int o = threadIdx.x; o < a.cout; o += blockDim.x)
        ws[nw + o] = a.bias ? bfv(a.bias[o]) : 0.0f;
    __syncthreads();
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)a.B * a.P) return;
    const int b = (int)(idx / a.P), p = (int)(idx % a.P);
    float acc[CO];
#pragma unroll
    for (int o = 0; o < CO; o++) acc[o] = o < a.cout ? ws[nw + o] : 0.0f;
    const float* src = a.in + (long long)b * a.in_bs + p;
    for (int i0 = 0; i0 < a.cin; i0 += 8) {
        float v[8];                        // eight independent loads in flight
#pragma unroll
        for (int j = 0; j < 8; j++) v[j] = i0 + j < a.cin ? src[(long long)(i0 + j) * a.P] : 0.0f;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            if (i0 + j >= a.cin) break;
            const float* wr = ws + (i0 + j) * a.cout;
#pragma unroll
            for (int o = 0; o < CO; o++)
                if (o < a.cout) acc[o] += wr[o] * v[j];
        }
    }
    const long long base = (long long)b * a.cout * a.P + p;
#pragma unroll
    for (int o = 0; o < CO; o++) {
        if (o >= a.cout) break;
        const long long k = base + (long long)o * a.P;
        float u = acc[o];
        if (a.add) u += a.add[k];
        if (a.pre) a.pre[k] = u;
        float z = u;
        if (a.film) z = u * (1.0f + a.film[(long long)b * a.fs + o]) + a.film[(long long)b * a.fs + a.cout + o];
        float r = z;
        if (a.act == 1) r = gelu(z);
        else if (a.act == 2) r = z * gelu_d(a.gate[k]);
        a.out[k] = a.accumulate ? a.out[k] + r : r;
    }
}

// Tensor-core helpers: mma.sync m16n8k8 TF32 and m16n8k16 bf16, fp32
// accumulation.  fp32 operands are split into a high part and the rounding
// of the remainder, and the partial products summed, so that the sums keep
// fp32-level accuracy.
__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void mma_tf32(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// (e0, e1) -> bf16 pairs (lower index in the low half): h = rn(e), l = rn(e - h)
__device__ __forceinline__ void split_bf16x2(float e0, float e1, uint32_t& h, uint32_t& l) {
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(h) : "f"(e1), "f"(e0));
    const float h0 = __uint_as_float(h << 16), h1 = __uint_as_float(h & 0xffff0000u);
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(l) : "f"(e1 - h1), "f"(e0 - h0));
}

// The channel mix on the tensor cores, for cout % 16 == 0 (cout <= 64) and
// P % 32 == 0 (cin padded to a multiple of 16 with zero weights and zero
// inputs): each warp takes 32 voxels of one sample and forms
// out[o][p] = sum_i W[o][i] in[i][p] with mma.sync m16n8k16 bf16, then runs
// the same epilogue as fno_pointwise.  The weights are bf16 already; each
// input is split into two bf16 parts (16 significant bits) and both
// products accumulated in fp32.
template <int MT>   // cout / 16
__global__ void __launch_bounds__(128) fno_pointwise_tc(PW a) {
    extern __shared__ uint32_t wp[];       // [cout][ci16 / 2 + 4] bf16 weight pairs, then [cout] bias
    const int ci16 = (a.cin + 15) & ~15;
    const int ldp = ci16 / 2 + 4;          // pairs per row: the A-fragment loads hit 32 banks
    for (int e = threadIdx.x; e < a.cout * (ci16 / 2); e += blockDim.x) {
        const int o = e / (ci16 / 2), i = 2 * (e % (ci16 / 2));
        uint32_t lo = 0, hi = 0;
        if (i < a.cin) lo = a.w[a.trans ? i * a.cout + o : o * a.cin + i];
        if (i + 1 < a.cin) hi = a.w[a.trans ? (i + 1) * a.cout + o : o * a.cin + i + 1];
        wp[o * ldp + e % (ci16 / 2)] = lo | (hi << 16);
    }
    float* bs = reinterpret_cast<float*>(wp + a.cout * ldp);
    for (int o = threadIdx.x; o < a.cout; o += blockDim.x) bs[o] = a.bias ? bfv(a.bias[o]) : 0.0f;
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const long long v0 = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31);
    if (v0 >= (long long)a.B * a.P) return;
    const int b = (int)(v0 / a.P), p0 = (int)(v0 % a.P);
    const float* src = a.in + (long long)b * a.in_bs + p0 + g;
    float c[MT][4][4];
#pragma unroll
    for (int mt = 0; mt < MT; mt++)
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int q = 0; q < 4; q++) c[mt][nt][q] = 0.0f;
    for (int i0 = 0; i0 < ci16; i0 += 16) {
        // B fragments: rows (2t, 2t+1) and (2t+8, 2t+9) of this K step, voxel column g
        uint32_t bh[4][2], bl[4][2];
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int ii = i0 + 2 * t + 8 * h;
                const float x0 = ii < a.cin ? src[(long long)ii * a.P + nt * 8] : 0.0f;
                const float x1 = ii + 1 < a.cin ? src[(long long)(ii + 1) * a.P + nt * 8] : 0.0f;
                split_bf16x2(x0, x1, bh[nt][h], bl[nt][h]);
            }
#pragma unroll
        for (int mt = 0; mt < MT; mt++) {
            const uint32_t* wr = wp + (mt * 16 + g) * ldp + i0 / 2 + t;
            const uint32_t a0 = wr[0], a1 = wr[8 * ldp], a2 = wr[4], a3 = wr[8 * ldp + 4];
#pragma unroll
            for (int nt = 0; nt < 4; nt++) {
                mma_bf16(c[mt][nt], a0, a1, a2, a3, bl[nt][0], bl[nt][1]);
                mma_bf16(c[mt][nt], a0, a1, a2, a3, bh[nt][0], bh[nt][1]);
            }
        }
    }
    // epilogue: accumulator q holds (o, p) = (16 mt + g + 8 (q >> 1), p0 + 8 nt + 2 t + (q & 1))
#pragma unroll
    for (int mt = 0; mt < MT; mt++)
#pragma unroll
        for (int r = 0; r < 2; r++) {
            const int o = mt * 16 + g + 8 * r;
            const float bo = bs[o];
            float f0 = 0.0f, f1 = 0.0f;
            if (a.film) {
                f0 = a.film[(long long)b * a.fs + o];
                f1 = a.film[(long long)b * a.fs + a.cout + o];
            }
#pragma unroll
            for (int nt = 0; nt < 4; nt++) {
                const long long k = ((long long)b * a.cout + o) * a.P + p0 + nt * 8 + 2 * t;
                float u[2] = {c[mt][nt][2 * r] + bo, c[mt][nt][2 * r + 1] + bo};
                if (a.add) {
                    const float2 ad = *reinterpret_cast<const float2*>(a.add + k);
                    u[0] += ad.x;
                    u[1] += ad.y;
                }
                if (a.pre) *reinterpret_cast<float2*>(a.pre + k) = make_float2(u[0], u[1]);
                float2 gt = make_float2(0.0f, 0.0f);
                if (a.act == 2) gt = *reinterpret_cast<const float2*>(a.gate + k);
                float rr[2];
#pragma unroll
                for (int j = 0; j < 2; j++) {
                    float z = u[j];
                    if (a.film) z = u[j] * (1.0f + f0) + f1;
                    float q = z;
                    if (a.act == 1) q = gelu(z);
                    else if (a.act == 2) q = z * gelu_d(j ? gt.y : gt.x);
                    rr[j] = q;
                }
                float2* op = reinterpret_cast<float2*>(a.out + k);
                if (a.accumulate) {
                    const float2 prev = *op;
                    rr[0] = prev.x + rr[0];
                    rr[1] = prev.y + rr[1];
                }
                *op = make_float2(rr[0], rr[1]);
            }
        }
}

// ---------------------------------------------------------------------------
// truncated 2-D DFTs (one CTA per channel plane)
// tw[k] = (cos 2 pi k / n, sin 2 pi k / n); mode q = kxi*m + ky
// ---------------------------------------------------------------------------
__device__ __forceinline__ int mode_kx(int kxi, int n, int m) { return kxi < m ? kxi : n - 2 * m + kxi; }

// F[plane][q] = s[ky] * sum_{x,y} f[plane][x*n+y] e^{-2 pi i (kx x + ky y) / n}
__global__ void fno_analysis(const float* in, float2* out, const float2* tw_g, const float* s_g,
                             int n, int m) {
    extern __shared__ float sm[];
    float* f = sm;                                  // n*n (padded to an even count)
    float2* A = reinterpret_cast<float2*>(f + ((n * n + 1) & ~1));  // n*m
    float2* tw = A + n * m;                         // n
    const int P = n * n, M = 2 * m * m;
    const long long plane = blockIdx.x;
    const float* src = in + plane * P;
    for (int e = threadIdx.x; e < P; e += blockDim.x) f[e] = src[e];
    for (int e = threadIdx.x; e < n; e += blockDim.x) tw[e] = tw_g[e];
    __syncthreads();
    for (int e = threadIdx.x; e < n * m; e += blockDim.x) {
        const int x = e / m, ky = e % m;
        float re = 0.0f, im = 0.0f;
        const float* row = f + x * n;
        int k = 0;                          // (ky * y) mod n
        for (int y = 0; y < n; y++) {
            const float2 t = tw[k];
            re += row[y] * t.x;
            im -= row[y] * t.y;
            k += ky;
            if (k >= n) k -= n;
        }
        A[x * m + ky] = make_float2(re, im);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < M; q += blockDim.x) {
        const int kxi = q / m, ky = q % m, kx = mode_kx(kxi, n, m);
        float re = 0.0f, im = 0.0f;
        int k = 0;                          // (kx * x) mod n
        for (int x = 0; x < n; x++) {
            const float2 a = A[x * m + ky];
            const float2 t = tw[k];
            re += a.x * t.x + a.y * t.y;
            im += a.y * t.x - a.x * t.y;
            k += kx;
            if (k >= n) k -= n;
        }
        const float sc = s_g[ky];
        out[plane * M + q] = make_float2(sc * re, sc * im);
    }
}

// f[plane][x*n+y] (=|+=) sum_q s[ky] Re(F[plane][q] e^{+2 pi i (kx x + ky y) / n})
__global__ void fno_synthesis(const float2* in, float* out, const float2* tw_g, const float* s_g,
                              int n, int m, int accumulate) {
    extern __shared__ float sm[];
    float2* F = reinterpret_cast<float2*>(sm);      // M
    float2* Z = F + 2 * m * m;                      // n*m
    float2* tw = Z + n * m;                         // n
    const int P = n * n, M = 2 * m * m;
    const long long plane = blockIdx.x;
    for (int e = threadIdx.x; e < M; e += blockDim.x) {
        const float2 v = in[plane * M + e];
        const float sc = s_g[e % m];
        F[e] = make_float2(sc * v.x, sc * v.y);
    }
    for (int e = threadIdx.x; e < n; e += blockDim.x) tw[e] = tw_g[e];
    __syncthreads();
    for (int e = threadIdx.x; e < n * m; e += blockDim.x) {
        const int x = e / m, ky = e % m;
        float re = 0.0f, im = 0.0f;
        int k = 0;                          // (kx * x) mod n, kx = 0, 1, .., m-1
        for (int kxi = 0; kxi < m; kxi++) {
            const float2 v = F[kxi * m + ky];
            const float2 t = tw[k];
            re += v.x * t.x - v.y * t.y;
            im += v.x * t.y + v.y * t.x;
            k += x;
            if (k >= n) k -= n;
        }
        k = ((n - m) * x) % n;              // kx = n-m, .., n-1
        for (int kxi = m; kxi < 2 * m; kxi++) {
            const float2 v = F[kxi * m + ky];
            const float2 t = tw[k];
            re += v.x * t.x - v.y * t.y;
            im += v.x * t.y + v.y * t.x;
            k += x;
            if (k >= n) k -= n;
        }
        Z[x * m + ky] = make_float2(re, im);
    }
    __syncthreads();
    float* dst = out + plane * P;
    for (int e = threadIdx.x; e < P; e += blockDim.x) {
        const int x = e / n, y = e % n;
        float r = 0.0f;
        int k = 0;                          // (ky * y) mod n
        for (int ky = 0; ky < m; ky++) {
            const float2 z = Z[x * m + ky];
            const float2 t = tw[k];
            r += z.x * t.x - z.y * t.y;
            k += y;
            if (k >= n) k -= n;
        }
        dst[e] = accumulate ? dst[e] + r : r;
    }
}

// The same truncated DFTs on the tensor cores, one warp per channel plane,
// for n % 16 == 0 and 2m <= 32 (n <= 64: at most 103 KB of shared memory).
// Each is two real GEMMs against twiddle matrices (fp32, computed in
// double) staged in shared memory, mma.sync m16n8k16 bf16 with both
// operands split into two bf16 parts (lo*hi + hi*lo + hi*hi in fp32):
//   analysis   R[x][c] = sum_y f[x][y] T1[y][c], c < m: cos, m <= c < 2m: -sin
//              (of 2 pi ky y / n); P[r][c] = sum_x T2[r][x] R[x][c], rows
//              r < 2m: cos, 2m <= r < 4m: sin (of 2 pi kx x / n); then
//              Re = P[kxi][ky] + P[2m+kxi][m+ky], Im = P[kxi][m+ky] - P[2m+kxi][ky]
//   synthesis  Z[x][c] = sum_k U[x][k] V[k][c] with U = T2 transposed and V
//              holding (Fr, Fi | -Fi, Fr) of the scaled modes, so Z = (Zr | Zi);
//              f[x][y] = sum_c Z[x][c] W[c][y] with W = T1 transposed.
// Padding rows and columns of the matrices are zero.  Row strides are chosen
// so that every fragment load from shared memory touches 32 banks: A
// fragments (float pairs at [g][2t]) want a stride of 8 mod 16 words, B
// fragments (rows 2t, 2t+1 at column g) 4 mod 8.
constexpr int kDftWarps = 4;

struct DftTc {
    int N2, K2, R4;   // 2m rounded up to 8 and to 16, 4m rounded up to 16
    int ld1, ld2;     // analysis T1 [y][c] (B), T2 [r][x] (A)
    int ldR, ldP;     // analysis per-warp R [x][c] (B), P [r][c]
    int ldU, ldW;     // synthesis U [x][k] (A), W [c][y] (B)
    int ldV, ldZ;     // synthesis per-warp V [k][c] (B), Z [x][c] (A)
};

__host__ __device__ inline DftTc dft_tc_layout(int n, int m) {
    DftTc L;
    L.N2 = (2 * m + 7) & ~7;
    L.K2 = (2 * m + 15) & ~15;
    L.R4 = (4 * m + 15) & ~15;
    L.ld1 = L.N2 + 4;
    L.ld2 = n + 8;
    L.ldR = L.N2 + 4;
    L.ldP = L.N2;
    L.ldU = L.R4 + 8;
    L.ldW = n + 4;
    L.ldV = L.N2 + 4;
    L.ldZ = L.K2 + 8;
    return L;
}

inline bool dft_tc_ok(int n, int m) { return n % 16 == 0 && 2 * m <= 32; }

inline size_t dft_tc_smem(int n, int m, bool synthesis) {
    const DftTc L = dft_tc_layout(n, m);
    const size_t fl = synthesis
        ? (size_t)n * L.ldU + (size_t)L.K2 * L.ldW + kDftWarps * ((size_t)L.R4 * L.ldV + (size_t)n * L.ldZ)
        : (size_t)n * L.ld1 + (size_t)L.R4 * L.ld2 + kDftWarps * ((size_t)n * L.ldR + (size_t)L.R4 * L.ldP);
    return sizeof(float) * fl;
}

// c += a * b with a, b given as (high, low) bf16 parts
__device__ __forceinline__ void mma3(float (&c)[4], const uint32_t (&ah)[4], const uint32_t (&al)[4],
                                     const uint32_t (&bh)[2], const uint32_t (&bl)[2]) {
    mma_bf16(c, al[0], al[1], al[2], al[3], bh[0], bh[1]);
    mma_bf16(c, ah[0], ah[1], ah[2], ah[3], bl[0], bl[1]);
    mma_bf16(c, ah[0], ah[1], ah[2], ah[3], bh[0], bh[1]);
}

// A fragment (16 x 16) of rows g, g + 8 and column pairs 2t, 2t + 8 from
// row-major p (stride ld, even), p pointing at [row g][column 2t]
__device__ __forceinline__ void frag_a(const float* p, int ld, uint32_t (&h)[4], uint32_t (&l)[4]) {
    const float2 u0 = *reinterpret_cast<const float2*>(p);
    const float2 u1 = *reinterpret_cast<const float2*>(p + 8 * ld);
    const float2 u2 = *reinterpret_cast<const float2*>(p + 8);
    const float2 u3 = *reinterpret_cast<const float2*>(p + 8 * ld + 8);
    split_bf16x2(u0.x, u0.y, h[0], l[0]);
    split_bf16x2(u1.x, u1.y, h[1], l[1]);
    split_bf16x2(u2.x, u2.y, h[2], l[2]);
    split_bf16x2(u3.x, u3.y, h[3], l[3]);
}

// B fragment (16 x 8) of row pairs 2t, 2t + 8 and column g from row-major
// [k][n] p (stride ld), p pointing at [row 2t][column g]
__device__ __forceinline__ void frag_b(const float* p, int ld, uint32_t (&h)[2], uint32_t (&l)[2]) {
    split_bf16x2(p[0], p[ld], h[0], l[0]);
    split_bf16x2(p[8 * ld], p[9 * ld], h[1], l[1]);
}

// the 16 x 8 accumulator tile (rows r0 + g, r0 + g + 8; columns c0 + 2t, + 1)
__device__ __forceinline__ void store_c(float* p, int ld, int r0, int c0, int g, int t,
                                        const float (&c)[4]) {
    float* q = p + (r0 + g) * ld + c0 + 2 * t;
    q[0] = c[0];
    q[1] = c[1];
    q[8 * ld] = c[2];
    q[8 * ld + 1] = c[3];
}

__global__ void __launch_bounds__(32 * kDftWarps) fno_analysis_tc(const float* in, float2* out,
                                                                   const float* tA1,
                                                                   const float* tA2,
                                                                   const float* s_g, int n,
                                                                   int m, int planes) {
    extern __shared__ float sd[];
    const DftTc L = dft_tc_layout(n, m);
    float* T1 = sd;                        // [n][ld1]
    float* T2 = T1 + n * L.ld1;            // [R4][ld2]
    float* scr = T2 + L.R4 * L.ld2;
    for (int e = threadIdx.x; e < n * L.N2; e += blockDim.x) T1[(e / L.N2) * L.ld1 + e % L.N2] = tA1[e];
    for (int e = threadIdx.x; e < L.R4 * n; e += blockDim.x) T2[(e / n) * L.ld2 + e % n] = tA2[e];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const long long plane = (long long)blockIdx.x * kDftWarps + warp;
    if (plane >= planes) return;
    float* R = scr + warp * (n * L.ldR + L.R4 * L.ldP);
    float* Pm = R + n * L.ldR;
    const float* f = in + plane * n * n;
    const int NT = L.N2 / 8;
    uint32_t ah[4], al[4], bh[2], bl[2];
    // R = f T1: M = n (x), K = n (y), N = N2 (c)
    for (int mt = 0; mt < n / 16; mt++) {
        float c[4][4] = {};
        for (int k0 = 0; k0 < n; k0 += 16) {
            frag_a(f + (mt * 16 + g) * n + k0 + 2 * t, n, ah, al);
#pragma unroll
            for (int nt = 0; nt < 4; nt++)
                if (nt < NT) {
                    frag_b(T1 + (k0 + 2 * t) * L.ld1 + nt * 8 + g, L.ld1, bh, bl);
                    mma3(c[nt], ah, al, bh, bl);
                }
        }
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
            if (nt < NT) store_c(R, L.ldR, mt * 16, nt * 8, g, t, c[nt]);
    }
    __syncwarp();
    // P = T2 R: M = R4 (r), K = n (x), N = N2 (c)
    for (int mt = 0; mt < L.R4 / 16; mt++) {
        float c[4][4] = {};
        for (int k0 = 0; k0 < n; k0 += 16) {
            frag_a(T2 + (mt * 16 + g) * L.ld2 + k0 + 2 * t, L.ld2, ah, al);
#pragma unroll
            for (int nt = 0; nt < 4; nt++)
                if (nt < NT) {
                    frag_b(R + (k0 + 2 * t) * L.ldR + nt * 8 + g, L.ldR, bh, bl);
                    mma3(c[nt], ah, al, bh, bl);
                }
        }
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
            if (nt < NT) store_c(Pm, L.ldP, mt * 16, nt * 8, g, t, c[nt]);
    }
    __syncwarp();
    const int M = 2 * m * m;
    float2* dst = out + plane * M;
    for (int q = lane; q < M; q += 32) {
        const int kxi = q / m, ky = q % m;
        const float re = Pm[kxi * L.ldP + ky] + Pm[(2 * m + kxi) * L.ldP + m + ky];
        const float im = Pm[kxi * L.ldP + m + ky] - Pm[(2 * m + kxi) * L.ldP + ky];
        const float sc = s_g[ky];
        dst[q] = make_float2(sc * re, sc * im);
    }
}

__global__ void __launch_bounds__(32 * kDftWarps) fno_synthesis_tc(const float2* in, float* out,
                                                                    const float* tS1,
                                                                    const float* tS2,
                                                                    const float* s_g, int n,
                                                                    int m, int planes,
                                                                    int accumulate) {
    extern __shared__ float sd[];
    const DftTc L = dft_tc_layout(n, m);
    float* U = sd;                         // [n][ldU]
    float* W = U + n * L.ldU;              // [K2][ldW]
    float* scr = W + L.K2 * L.ldW;
    for (int e = threadIdx.x; e < n * L.R4; e += blockDim.x) U[(e / L.R4) * L.ldU + e % L.R4] = tS1[e];
    for (int e = threadIdx.x; e < L.K2 * n; e += blockDim.x) W[(e / n) * L.ldW + e % n] = tS2[e];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const long long plane = (long long)blockIdx.x * kDftWarps + warp;
    if (plane >= planes) return;
    float* V = scr + warp * (L.R4 * L.ldV + n * L.ldZ);
    float* Z = V + L.R4 * L.ldV;
    const int M = 2 * m * m, NT = L.N2 / 8;
    for (int e = lane; e < L.R4 * L.ldV; e += 32) V[e] = 0.0f;
    for (int e = lane; e < n * (L.K2 - L.N2); e += 32)    // Z's padding columns
        Z[(e / (L.K2 - L.N2)) * L.ldZ + L.N2 + e % (L.K2 - L.N2)] = 0.0f;
    __syncwarp();
    const float2* src = in + plane * M;
    for (int q = lane; q < M; q += 32) {
        const int kxi = q / m, ky = q % m;
        const float2 v = src[q];
        const float sc = s_g[ky];
        const float vr = sc * v.x, vi = sc * v.y;
        V[kxi * L.ldV + ky] = vr;
        V[kxi * L.ldV + m + ky] = vi;
        V[(2 * m + kxi) * L.ldV + ky] = -vi;
        V[(2 * m + kxi) * L.ldV + m + ky] = vr;
    }
    __syncwarp();
    uint32_t ah[4], al[4], bh[2], bl[2];
    // Z = U V: M = n (x), K = R4 (k), N = N2 (c); columns N2..K2 of Z stay zero
    for (int mt = 0; mt < n / 16; mt++) {
        float c[4][4] = {};
        for (int k0 = 0; k0 < L.R4; k0 += 16) {
            frag_a(U + (mt * 16 + g) * L.ldU + k0 + 2 * t, L.ldU, ah, al);
#pragma unroll
            for (int nt = 0; nt < 4; nt++)
                if (nt < NT) {
                    frag_b(V + (k0 + 2 * t) * L.ldV + nt * 8 + g, L.ldV, bh, bl);
                    mma3(c[nt], ah, al, bh, bl);
                }
        }
#pragma unroll
        for (int nt = 0; nt < 4; nt++)
            if (nt < NT) store_c(Z, L.ldZ, mt * 16, nt * 8, g, t, c[nt]);
    }
    __syncwarp();
    // f = Z W: M = n (x), K = K2 (c), N = n (y), two column tiles at a time
    float* dst = out + plane * n * n;
    for (int mt = 0; mt < n / 16; mt++)
        for (int nt0 = 0; nt0 < n / 8; nt0 += 2) {
            float c[2][4] = {};
            for (int k0 = 0; k0 < L.K2; k0 += 16) {
                frag_a(Z + (mt * 16 + g) * L.ldZ + k0 + 2 * t, L.ldZ, ah, al);
#pragma unroll
                for (int j = 0; j < 2; j++) {
                    frag_b(W + (k0 + 2 * t) * L.ldW + (nt0 + j) * 8 + g, L.ldW, bh, bl);
                    mma3(c[j], ah, al, bh, bl);
                }
            }
#pragma unroll
            for (int j = 0; j < 2; j++)
#pragma unroll
                for (int r = 0; r < 2; r++) {
                    float2* q = reinterpret_cast<float2*>(dst + (mt * 16 + g + 8 * r) * n +
                                                          (nt0 + j) * 8 + 2 * t);
                    float2 v = make_float2(c[j][2 * r], c[j][2 * r + 1]);
                    if (accumulate) {
                        const float2 o = *q;
                        v.x = o.x + v.x;
                        v.y = o.y + v.y;
                    }
                    *q = v;
                }
        }
}

// ---------------------------------------------------------------------------
// per-mode channel mixing (one CTA per mode q)
// conj_t = 0: Y[b][o][q] = sum_i X[b][i][q] W[q][i][o]
// conj_t = 1: Y[b][i][q] = sum_o X[b][o][q] conj(W[q][i][o])
// ---------------------------------------------------------------------------
__global__ void fno_mix(const float2* X, const uint16_t* w, float2* Y, int B, int C, int M,
                        int conj_t) {
    extern __shared__ float2 wsm[];                 // [in][out] after transposition
    const int q = blockIdx.x;
    const uint16_t* wq = w + (long long)q * C * C * 2;
    for (int e = threadIdx.x; e < C * C; e += blockDim.x) {
        const int i = e / C, o = e % C;
        const float re = bfv(wq[2 * e]), im = bfv(wq[2 * e + 1]);
        if (conj_t) wsm[o * C + i] = make_float2(re, -im);
        else        wsm[i * C + o] = make_float2(re, im);
    }
    float2* xs = wsm + C * C;               // [16][C] inputs of this mode
    for (int b0 = 0; b0 < B; b0 += 16) {
        const int nb = min(16, B - b0);
        __syncthreads();
        for (int e = threadIdx.x; e < nb * C; e += blockDim.x)
            xs[e] = X[((long long)b0 * C + e) * M + q];
        __syncthreads();
        for (int e = threadIdx.x; e < nb * C; e += blockDim.x) {
            const int bb = e / C, o = e % C;
            float re = 0.0f, im = 0.0f;
            const float2* xr = xs + bb * C;
            for (int i = 0; i < C; i++) {
                const float2 x = xr[i];
                const float2 ww = wsm[i * C + o];
                re += x.x * ww.x - x.y * ww.y;
                im += x.x * ww.y + x.y * ww.x;
            }
            Y[((long long)(b0 + bb) * C + o) * M + q] = make_float2(re, im);
        }
    }
}

// The per-mode mix on the tensor cores (C = 16, 32 or 64): with the
// inputs of 64 samples as real rows [Re X | Im X] (K = 2C) and the complex
// (in, out) matrix Wc in real form B = [[Re, Im], [-Im, Re]] (2C x 2C, bf16
// exact), [Re Y | Im Y] = X B.  One CTA per mode, warp w takes samples
// 16w .. 16w + 15 and all 2C output columns; mma.sync m16n8k16 bf16 with
// the inputs split into two bf16 parts.  B is kept transposed as bf16 pairs
// along K, so a B fragment is two 32-bit loads.
template <int C>
__global__ void __launch_bounds__(128) fno_mix_tc(const float2* X, const uint16_t* w, float2* Y,
                                                  int B, int M, int conj_t) {
    constexpr int K2 = 2 * C, NT = K2 / 8;
    constexpr int LDB = C + 4;             // pairs per row of Bt: B-fragment loads hit 32 banks
    constexpr int LDX = K2 + 8;            // floats per row of Xs: A-fragment float2 loads too
    extern __shared__ uint32_t smx[];
    uint32_t* Bt = smx;                                      // [K2 (n)][LDB] pairs along k
    float* Xs = reinterpret_cast<float*>(smx + K2 * LDB);    // [64][LDX]
    const int q = blockIdx.x;
    const uint16_t* wq = w + (long long)q * C * C * 2;
    for (int e = threadIdx.x; e < K2 * C; e += blockDim.x) {
        const int n = e / C, kp = e % C;
        uint32_t pr = 0;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int k = 2 * kp + h, i = k % C, o = n % C;
            // Wc[i][o] = W[i][o], or conj(W[o][i]) for the conjugate transpose
            const int src = conj_t ? o * C + i : i * C + o;
            const float re = bfv(wq[2 * src]);
            const float im = conj_t ? -bfv(wq[2 * src + 1]) : bfv(wq[2 * src + 1]);
            const float v = k < C ? (n < C ? re : im) : (n < C ? -im : re);
            pr |= (uint32_t)to_bf16(v) << (16 * h);
        }
        Bt[n * LDB + kp] = pr;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    for (int b0 = 0; b0 < B; b0 += 64) {
        const int nb = min(64, B - b0);
        __syncthreads();
        for (int e = threadIdx.x; e < 64 * C; e += blockDim.x) {
            const int bb = e / C, c = e % C;
            float2 v = make_float2(0.0f, 0.0f);
            if (bb < nb) v = X[((long long)(b0 + bb) * C + c) * M + q];
            Xs[bb * LDX + c] = v.x;
            Xs[bb * LDX + C + c] = v.y;
        }
        __syncthreads();
        float acc[NT][4];
#pragma unroll
        for (int nt = 0; nt < NT; nt++)
#pragma unroll
            for (int r = 0; r < 4; r++) acc[nt][r] = 0.0f;
#pragma unroll
        for (int k0 = 0; k0 < K2; k0 += 16) {
            uint32_t ah[4], al[4];
            frag_a(Xs + (warp * 16 + g) * LDX + k0 + 2 * t, LDX, ah, al);
#pragma unroll
            for (int nt = 0; nt < NT; nt++) {
                const uint32_t* bp = Bt + (nt * 8 + g) * LDB + k0 / 2 + t;
                const uint32_t b0r = bp[0], b1r = bp[4];
                mma_bf16(acc[nt], al[0], al[1], al[2], al[3], b0r, b1r);
                mma_bf16(acc[nt], ah[0], ah[1], ah[2], ah[3], b0r, b1r);
            }
        }
        // column o (< C) of tile nt holds Re Y, the same column of tile nt + NT/2 Im Y
#pragma unroll
        for (int nt = 0; nt < NT / 2; nt++)
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const int bb = warp * 16 + g + 8 * r;
                if (bb >= nb) continue;
#pragma unroll
                for (int j = 0; j < 2; j++) {
                    const int o = nt * 8 + 2 * t + j;
                    Y[((long long)(b0 + bb) * C + o) * M + q] =
                        make_float2(acc[nt][2 * r + j], acc[nt + NT / 2][2 * r + j]);
                }
            }
    }
}

// Its weight gradient on the tensor cores (C = 16 or 32): P = A D with
// A[i'][b] = [Re X; Im X] (2C x samples) and D[b][n'] = [Re dY | Im dY],
// then dW re = P[i][o] + P[C+i][C+o], im = P[i][C+o] - P[C+i][o].  Each work
// unit is the four 16 x 8 tiles (mt, nt), (mt, nt + C/8), (mt + C/16, nt),
// (mt + C/16, nt + C/8) that one output block needs; samples in chunks of
// 64, both operands split into two bf16 parts (3 products).
template <int C>
__global__ void __launch_bounds__(128) fno_mix_wgrad_tc(const float2* X, const float2* dY,
                                                        float* gw, int B, int M) {
    constexpr int K2 = 2 * C, MP = C / 16, NP = C / 8, UNITS = MP * NP, UPW = (UNITS + 3) / 4;
    constexpr int LDA = 64 + 8, LDY = K2 + 4;
    extern __shared__ float smw[];
    float* Xt = smw;                 // [K2][LDA]
    float* Ys = smw + K2 * LDA;      // [64][LDY]
    const int q = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float acc[UPW][4][4];
#pragma unroll
    for (int u = 0; u < UPW; u++)
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int r = 0; r < 4; r++) acc[u][a][r] = 0.0f;
    for (int b0 = 0; b0 < B; b0 += 64) {
        const int nb = min(64, B - b0);
        __syncthreads();
        for (int e = threadIdx.x; e < 64 * C; e += blockDim.x) {
            const int bb = e / C, c = e % C;
            float2 x = make_float2(0.0f, 0.0f), y = make_float2(0.0f, 0.0f);
            if (bb < nb) {
                const long long k = ((long long)(b0 + bb) * C + c) * M + q;
                x = X[k];
                y = dY[k];
            }
            Xt[c * LDA + bb] = x.x;
            Xt[(C + c) * LDA + bb] = x.y;
            Ys[bb * LDY + c] = y.x;
            Ys[bb * LDY + C + c] = y.y;
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < UPW; u++) {
            const int unit = warp + 4 * u;
            if (unit >= UNITS) break;
            const int mt = unit / NP, nt = unit % NP;
#pragma unroll
            for (int k0 = 0; k0 < 64; k0 += 16) {
                uint32_t ah0[4], al0[4], ah1[4], al1[4], bh0[2], bl0[2], bh1[2], bl1[2];
                frag_a(Xt + (mt * 16 + g) * LDA + k0 + 2 * t, LDA, ah0, al0);
                frag_a(Xt + ((mt + MP) * 16 + g) * LDA + k0 + 2 * t, LDA, ah1, al1);
                frag_b(Ys + (k0 + 2 * t) * LDY + nt * 8 + g, LDY, bh0, bl0);
                frag_b(Ys + (k0 + 2 * t) * LDY + (nt + NP) * 8 + g, LDY, bh1, bl1);
                mma3(acc[u][0], ah0, al0, bh0, bl0);
                mma3(acc[u][1], ah0, al0, bh1, bl1);
                mma3(acc[u][2], ah1, al1, bh0, bl0);
                mma3(acc[u][3], ah1, al1, bh1, bl1);
            }
        }
    }
    float* gq = gw + (long long)q * C * C * 2;
#pragma unroll
    for (int u = 0; u < UPW; u++) {
        const int unit = warp + 4 * u;
        if (unit >= UNITS) break;
        const int mt = unit / NP, nt = unit % NP;
#pragma unroll
        for (int r = 0; r < 2; r++)
#pragma unroll
            for (int j = 0; j < 2; j++) {
                const int i = mt * 16 + g + 8 * r, o = nt * 8 + 2 * t + j, a = 2 * r + j;
                gq[2 * (i * C + o)] = acc[u][0][a] + acc[u][3][a];
                gq[2 * (i * C + o) + 1] = acc[u][1][a] - acc[u][2][a];
            }
    }
}

// dW[q][i][o] = sum_b conj(X[b][i][q]) dY[b][o][q], written as fp32 pairs
__global__ void fno_mix_wgrad(const float2* X, const float2* dY, float* gw, int B, int C, int M) {
    extern __shared__ float2 sm2[];
    constexpr int BC = 16;
    float2* xs = sm2;               // [BC][C]
    float2* ys = sm2 + BC * C;      // [BC][C]
    const int q = blockIdx.x;
    // pairs (i, o) = threadIdx.x + r * 256, r < 16 (C <= 64)
    float accr[16], acci[16];
#pragma unroll
    for (int r = 0; r < 16; r++) { accr[r] = 0.0f; acci[r] = 0.0f; }
    for (int b0 = 0; b0 < B; b0 += BC) {
        const int nb = min(BC, B - b0);
        __syncthreads();
        for (int e = threadIdx.x; e < nb * C; e += blockDim.x) {
            const int bb = e / C, c = e % C;
            const long long k = ((long long)(b0 + bb) * C + c) * M + q;
            xs[bb * C + c] = X[k];
            ys[bb * C + c] = dY[k];
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < 16; r++) {
            const int e = threadIdx.x + r * 256;
            if (e >= C * C) break;
            const int i = e / C, o = e % C;
            float re = accr[r], im = acci[r];
            for (int bb = 0; bb < nb; bb++) {
                const float2 x = xs[bb * C + i], y = ys[bb * C + o];
                re += x.x * y.x + x.y * y.y;     // conj(x) * y
                im += x.x * y.y - x.y * y.x;
            }
            accr[r] = re;
            acci[r] = im;
        }
    }
    float* g = gw + (long long)q * C * C * 2;
#pragma unroll
    for (int r = 0; r < 16; r++) {
        const int e = threadIdx.x + r * 256;
        if (e >= C * C) break;
        g[2 * e] = accr[r];
        g[2 * e + 1] = acci[r];
    }
}

// ---------------------------------------------------------------------------
// pointwise weight gradients: dW[o][i] = sum_{b,p} dY[b][o][p] X[b][i][p],
// db[o] = sum dY.  Partial sums per (sample, tile of kTile voxels), then an
// ordered reduction over the tiles.
// ---------------------------------------------------------------------------
// The weight products run on the tensor cores: the tile's dY rows (A, O
// padded to 16) and x rows (B, I padded to 8) are staged in shared memory,
// each warp takes 16 x 8 output tiles, mma.sync m16n8k8 TF32 over the
// tile's 128 voxels.  Both operands are split into TF32 high and low parts
// and lo*hi + hi*lo + hi*hi accumulated in fp32 (fp32-level accuracy).
// Partial rows: [O*I weights, O biases] per CTA.
constexpr int kLdTc = kTile + 4;   // row pad: fragment loads hit 32 banks

__global__ void __launch_bounds__(256) fno_wgrad_partial_tc(const float* dy, const float* x,
                                                            long long x_bs, int O, int I, int P,
                                                            int tiles, float* part) {
    extern __shared__ float sm[];
    const int Op = (O + 15) & ~15, Ip = (I + 7) & ~7;
    float* ys = sm;                  // [Op][kLdTc]
    float* xs = sm + Op * kLdTc;     // [Ip][kLdTc]
    const int b = blockIdx.x / tiles, tt = blockIdx.x % tiles;
    const int p0 = tt * kTile;
    for (int e = threadIdx.x; e < Op * kTile; e += blockDim.x) {
        const int o = e / kTile, pp = e % kTile, p = p0 + pp;
        ys[o * kLdTc + pp] = (o < O && p < P) ? dy[((long long)b * O + o) * P + p] : 0.0f;
    }
    for (int e = threadIdx.x; e < Ip * kTile; e += blockDim.x) {
        const int i = e / kTile, pp = e % kTile, p = p0 + pp;
        xs[i * kLdTc + pp] = (i < I && p < P) ? x[(long long)b * x_bs + (long long)i * P + p] : 0.0f;
    }
    __syncthreads();
    float* dst = part + (long long)blockIdx.x * (O * I + O);
    for (int o = threadIdx.x; o < O; o += blockDim.x) {
        const float* yr = ys + o * kLdTc;
        float s = 0.0f;
        for (int pp = 0; pp < kTile; pp++) s += yr[pp];
        dst[O * I + o] = s;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int ntl = Ip / 8, ntiles = (Op / 16) * ntl;
    for (int tile = warp; tile < ntiles; tile += (int)(blockDim.x >> 5)) {
        const int mt = tile / ntl, nt = tile % ntl;
        const float* ar = ys + (mt * 16 + g) * kLdTc + t;
        const float* br = xs + (nt * 8 + g) * kLdTc + t;
        float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 4
        for (int k0 = 0; k0 < kTile; k0 += 8) {
            const float av[4] = {ar[k0], ar[k0 + 8 * kLdTc], ar[k0 + 4], ar[k0 + 8 * kLdTc + 4]};
            const float bv[2] = {br[k0], br[k0 + 4]};
            uint32_t ah[4], al[4], bh[2], bl[2];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                ah[q] = to_tf32(av[q]);
                al[q] = to_tf32(av[q] - __uint_as_float(ah[q]));
            }
#pragma unroll
            for (int q = 0; q < 2; q++) {
                bh[q] = to_tf32(bv[q]);
                bl[q] = to_tf32(bv[q] - __uint_as_float(bh[q]));
            }
            mma_tf32(c, al[0], al[1], al[2], al[3], bh[0], bh[1]);
            mma_tf32(c, ah[0], ah[1], ah[2], ah[3], bl[0], bl[1]);
            mma_tf32(c, ah[0], ah[1], ah[2], ah[3], bh[0], bh[1]);
        }
        const int o = mt * 16 + g, i = nt * 8 + 2 * t;
#pragma unroll
        for (int r = 0; r < 2; r++)
            if (o + 8 * r < O) {
                if (i < I) dst[(o + 8 * r) * I + i] = c[2 * r];
                if (i + 1 < I) dst[(o + 8 * r) * I + i + 1] = c[2 * r + 1];
            }
    }
}

// 256 threads: 32 consecutive entries (lanes) x 8 groups of partial rows,
// combined in a fixed order
__global__ void fno_wgrad_reduce(const float* part, int nblk, int O, int I, float* gw, float* gb) {
    __shared__ float red[8][33];
    const int E = O * I + O;
    const int lane = threadIdx.x & 31, grp = threadIdx.x >> 5;
    const int e = blockIdx.x * 32 + lane;
    float s = 0.0f;
    if (e < E)
        for (int c = grp; c < nblk; c += 8) s += part[(long long)c * E + e];
    red[grp][lane] = s;
    __syncthreads();
    if (grp == 0 && e < E) {
        float t = red[0][lane];
        for (int g = 1; g < 8; g++) t += red[g][lane];
        if (e < O * I) gw[e] = t;
        else gb[e - O * I] = t;
    }
}

// ---------------------------------------------------------------------------
// FiLM + GELU backward, one CTA per (sample, channel) plane of layer k:
// z = u (1 + g0) + g1, h' = GELU(z); du = dh' GELU'(z) (1 + g0),
// dg0 = sum dh' GELU'(z) u, dg1 = sum dh' GELU'(z)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float block_sum(float v, float* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    float s = 0.0f;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += red[k];
    return s;   // valid in thread 0
}

__global__ void fno_film_back(const float* dh, const float* u, const float* g, int C, int P,
                              int gs, int k, float* du, float* dg) {
    __shared__ float red[32];
    const int b = blockIdx.x / C, o = blockIdx.x % C;
    const float g0 = g[(long long)b * gs + 2 * k * C + o];
    const float g1 = g[(long long)b * gs + 2 * k * C + C + o];
    const long long base = ((long long)b * C + o) * P;
    float s0 = 0.0f, s1 = 0.0f;
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        const float uu = u[base + p];
        const float z = uu * (1.0f + g0) + g1;
        const float dz = dh[base + p] * gelu_d(z);
        du[base + p] = dz * (1.0f + g0);
        s0 += dz * uu;
        s1 += dz;
    }
    s0 = block_sum(s0, red);
    s1 = block_sum(s1, red);
    if (threadIdx.x == 0) {
        dg[(long long)b * gs + 2 * k * C + o] = s0;
        dg[(long long)b * gs + 2 * k * C + C + o] = s1;
    }
}

// ---------------------------------------------------------------------------
// conditioning MLP (rows of the batch)
// ---------------------------------------------------------------------------
// out[b][j] = act(sum_k W[j][k] in[b][k] + bias[j]); pre (if set) before act
__global__ void fno_dense(const float* in, int K, const uint16_t* w, const uint16_t* bias, int J,
                          int B, int act, float* pre, float* out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= B * J) return;
    const int b = e / J, j = e % J;
    float s = bfv(bias[j]);
    for (int k = 0; k < K; k++) s += bfv(w[j * K + k]) * in[b * K + k];
    if (pre) pre[e] = s;
    out[e] = act ? gelu(s) : s;
}

// dW[j][k] = sum_b d[b][j] in[b][k], db[j] = sum_b d[b][j]
__global__ void fno_dense_wgrad(const float* d, const float* in, int B, int J, int K, float* gw,
                                float* gb) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= J * K + J) return;
    float s = 0.0f;
    if (e < J * K) {
        const int j = e / K, k = e % K;
        for (int b = 0; b < B; b++) s += d[b * J + j] * in[b * K + k];
        gw[e] = s;
    } else {
        const int j = e - J * K;
        for (int b = 0; b < B; b++) s += d[b * J + j];
        gb[j] = s;
    }
}

// din[b][k] = (sum_j W[j][k] d[b][j]) * GELU'(gate[b][k])
__global__ void fno_dense_dinput(const float* d, const uint16_t* w, int B, int J, int K,
                                 const float* gate, float* din) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= B * K) return;
    const int b = e / K, k = e % K;
    float s = 0.0f;
    for (int j = 0; j < J; j++) s += bfv(w[j * K + k]) * d[b * J + j];
    din[e] = s * gelu_d(gate[e]);
}

// ---------------------------------------------------------------------------
// loss, gather, Adam
// ---------------------------------------------------------------------------
__global__ void fno_mse(const float* out, const float* y, long long N, float scale, float* dout,
                        float* part) {
    __shared__ float red[32];
    float s = 0.0f;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < N;
         e += (long long)gridDim.x * blockDim.x) {
        const float d = out[e] - y[e];
        dout[e] = scale * d;
        s += d * d;
    }
    s = block_sum(s, red);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void fno_mse_final(const float* part, int n, float inv_n, float* loss) {
    __shared__ float red[32];
    float s = 0.0f;
    for (int e = threadIdx.x; e < n; e += blockDim.x) s += part[e];
    s = block_sum(s, red);
    if (threadIdx.x == 0) loss[0] = s * inv_n;
}

__global__ void fno_gather(const float* src, const int* idx, int rows, long long R, float* dst) {
    const long long total = (long long)rows * R;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long r = e / R, c = e % R;
        dst[e] = src[(long long)idx[r] * R + c];
    }
}

// hyper: lr / (1 - beta1^t), sqrt(1 - beta2^t), beta1, beta2, eps
__global__ void fno_adam(float* p, uint16_t* pb, const float* g, float* m, float* v, long long n,
                         const float* hyper) {
    const float step = hyper[0], bc2s = hyper[1], b1 = hyper[2], b2 = hyper[3], eps = hyper[4];
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const float gg = g[e];
        const float mm = b1 * m[e] + (1.0f - b1) * gg;
        const float vv = b2 * v[e] + (1.0f - b2) * gg * gg;
        m[e] = mm;
        v[e] = vv;
        const float pp = p[e] - step * (mm / (sqrtf(vv) / bc2s + eps));
        p[e] = pp;
        pb[e] = to_bf16(pp);
    }
}

__global__ void fno_to_bf16(const float* p, uint16_t* pb, long long n) {
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x)
        pb[e] = to_bf16(p[e]);
}

}  // namespace fno
}  // namespace spg

// ===========================================================================
// host side
// ===========================================================================
using namespace spg::fno;

struct FnoOffsets {
    long long lift_w, lift_b, film1_w, film1_b, film2_w, film2_b, proj1_w, proj1_b, proj2_w,
        proj2_b, total;
    std::vector<long long> spec, lin_w, lin_b;
};

struct sp_fno {
    sp_fno_shape s{};
    FnoOffsets off;
    int P = 0, M = 0, G = 0;     // voxels, kept modes, FiLM outputs
    std::string err;
    cudaStream_t st = nullptr;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    std::vector<void*> allocs;
    // parameters
    float *p = nullptr, *grad = nullptr, *am = nullptr, *av = nullptr, *hyper = nullptr;
    uint16_t* pb = nullptr;
    float2* tw = nullptr;
    float *s_one = nullptr, *s_inv = nullptr;
    // twiddle matrices of the tensor-core DFTs (null when the shape does not fit them)
    float *tA1 = nullptr, *tA2 = nullptr, *tS1 = nullptr, *tS2 = nullptr;
    // activations [layers+1] h, [layers] u, [layers] X
    float *h = nullptr, *u = nullptr, *sbuf = nullptr, *q = nullptr, *a = nullptr;
    float2 *X = nullptr, *Y = nullptr;
    float *g = nullptr, *hid_pre = nullptr, *hid = nullptr;
    float* out = nullptr;        // the training step's output
    // backward
    float *dout = nullptr, *dq = nullptr, *dhA = nullptr, *dhB = nullptr, *du = nullptr;
    float2 *dY = nullptr, *dX = nullptr;
    float *dg = nullptr, *dhid = nullptr, *part = nullptr, *loss_part = nullptr, *loss = nullptr;
    // training-step staging
    float *cond_b = nullptr, *target_b = nullptr, *x_b = nullptr;
    int* idx_d = nullptr;
    int32_t* idx_h = nullptr;    // pinned
    float* hyper_h = nullptr;    // pinned
    long long adam_t = 0;
    // state of the last forward
    const float* last_x = nullptr;
    long long last_x_bs = 0;
    const float* last_cond = nullptr;
    float* last_out = nullptr;
    int last_batch = 0;
    // graphs of the training step, keyed by their arguments
    struct Graph {
        cudaGraphExec_t exec = nullptr;
        const float *x = nullptr, *cond = nullptr, *target = nullptr;
        int x_shared = 0, batch = 0;
    };
    std::vector<Graph> graphs;
};

namespace {

int fail(sp_fno* f, int code, const std::string& m) {
    if (f) f->err = m;
    return code;
}

int cuda_fail(sp_fno* f, cudaError_t e, const char* where) {
    return fail(f, SP_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

template <typename T>
T* dalloc(sp_fno* f, size_t count, bool& ok) {
    void* ptr = nullptr;
    if (!ok) return nullptr;
    if (cudaMalloc(&ptr, count * sizeof(T) + 16) != cudaSuccess) {
        ok = false;
        return nullptr;
    }
    f->allocs.push_back(ptr);
    return static_cast<T*>(ptr);
}

FnoOffsets offsets(const sp_fno_shape& s) {
    FnoOffsets o;
    const long long C = s.width, M = 2LL * s.modes * s.modes, H = s.hidden;
    long long k = 0;
    o.lift_w = k; k += C * s.in_ch;
    o.lift_b = k; k += C;
    for (int l = 0; l < s.layers; l++) {
        o.spec.push_back(k); k += M * C * C * 2;
        o.lin_w.push_back(k); k += C * C;
        o.lin_b.push_back(k); k += C;
    }
    const long long G = 2LL * s.layers * C;
    o.film1_w = k; k += H * s.cond;
    o.film1_b = k; k += H;
    o.film2_w = k; k += G * H;
    o.film2_b = k; k += G;
    o.proj1_w = k; k += H * C;
    o.proj1_b = k; k += H;
    o.proj2_w = k; k += (long long)s.out_ch * H;
    o.proj2_b = k; k += s.out_ch;
    o.total = k;
    return o;
}

long long fieldC(const sp_fno* f) { return (long long)f->s.max_batch * f->s.width * f->P; }

// ---- launch helpers --------------------------------------------------------
void pointwise(sp_fno* f, PW a) {
    const int tb = 128;
    const long long n = (long long)a.B * a.P;
    const size_t smem = sizeof(float) * (a.cin * a.cout + a.cout);
    const int nb = (int)((n + tb - 1) / tb);
    if (a.cout % 16 == 0 && a.cout <= 64 && a.cin <= 64 && a.P % 32 == 0) {
        const size_t tsm = sizeof(uint32_t) * (a.cout * (((a.cin + 15) & ~15) / 2 + 4) + a.cout);
        switch (a.cout / 16) {
            case 1: fno_pointwise_tc<1><<<nb, tb, tsm, f->st>>>(a); break;
            case 2: fno_pointwise_tc<2><<<nb, tb, tsm, f->st>>>(a); break;
            case 3: fno_pointwise_tc<3><<<nb, tb, tsm, f->st>>>(a); break;
            default: fno_pointwise_tc<4><<<nb, tb, tsm, f->st>>>(a); break;
        }
        return;
    }
    if (a.cout <= 8) fno_pointwise<8><<<nb, tb, smem, f->st>>>(a);
    else if (a.cout <= 16) fno_pointwise<16><<<nb, tb, smem, f->st>>>(a);
    else if (a.cout <= 32) fno_pointwise<32><<<nb, tb, smem, f->st>>>(a);
    else fno_pointwise<64><<<nb, tb, smem, f->st>>>(a);
}

PW pw_base(const sp_fno* f, int B) {
    PW a{};
    a.P = f->P;
    a.B = B;
    return a;
}

void analysis(sp_fno* f, const float* in, float2* out, int planes, const float* scale) {
    const int n = f->s.n, m = f->s.modes;
    if (f->tA1) {
        fno_analysis_tc<<<(planes + kDftWarps - 1) / kDftWarps, 32 * kDftWarps,
                          dft_tc_smem(n, m, false), f->st>>>(in, out, f->tA1, f->tA2, scale, n, m,
                                                            planes);
        return;
    }
    const size_t smem = sizeof(float) * ((n * n + 1) & ~1) + sizeof(float2) * (n * m + n);
    fno_analysis<<<planes, 256, smem, f->st>>>(in, out, f->tw, scale, n, m);
}

void synthesis(sp_fno* f, const float2* in, float* out, int planes, const float* scale, int acc) {
    const int n = f->s.n, m = f->s.modes;
    if (f->tS1) {
        fno_synthesis_tc<<<(planes + kDftWarps - 1) / kDftWarps, 32 * kDftWarps,
                           dft_tc_smem(n, m, true), f->st>>>(in, out, f->tS1, f->tS2, scale, n, m,
                                                            planes, acc);
        return;
    }
    const size_t smem = sizeof(float2) * (2 * m * m + n * m + n);
    fno_synthesis<<<planes, 256, smem, f->st>>>(in, out, f->tw, scale, n, m, acc);
}

void wgrad(sp_fno* f, const float* dy, const float* x, long long x_bs, int O, int I, int B,
           float* gw, float* gb) {
    const int tiles = (f->P + kTile - 1) / kTile;
    const int nblk = B * tiles;
    const size_t smem = sizeof(float) * (((O + 15) & ~15) + ((I + 7) & ~7)) * kLdTc;
    fno_wgrad_partial_tc<<<nblk, 256, smem, f->st>>>(dy, x, x_bs, O, I, f->P, tiles, f->part);
    const int E = O * I + O;
    fno_wgrad_reduce<<<(E + 31) / 32, 256, 0, f->st>>>(f->part, nblk, O, I, gw, gb);
}

inline size_t mix_tc_smem(int C) {
    return sizeof(uint32_t) * (2 * C * (C + 4) + 64 * (2 * C + 8));
}
inline size_t mix_wgrad_tc_smem(int C) {
    return sizeof(float) * (2 * C * (64 + 8) + 64 * (2 * C + 4));
}

void mix(sp_fno* f, const float2* X, const uint16_t* w, float2* Y, int B, int conj_t) {
    const int C = f->s.width, M = f->M;
    switch (C) {
        case 16: fno_mix_tc<16><<<M, 128, mix_tc_smem(16), f->st>>>(X, w, Y, B, M, conj_t); return;
        case 32: fno_mix_tc<32><<<M, 128, mix_tc_smem(32), f->st>>>(X, w, Y, B, M, conj_t); return;
        case 64: fno_mix_tc<64><<<M, 128, mix_tc_smem(64), f->st>>>(X, w, Y, B, M, conj_t); return;
        default: break;
    }
    const size_t msm = sizeof(float2) * (C * C + 16 * C);
    fno_mix<<<M, 256, msm, f->st>>>(X, w, Y, B, C, M, conj_t);
}

void mix_wgrad(sp_fno* f, const float2* X, const float2* dY, float* gw, int B) {
    const int C = f->s.width, M = f->M;
    switch (C) {
        case 16: fno_mix_wgrad_tc<16><<<M, 128, mix_wgrad_tc_smem(16), f->st>>>(X, dY, gw, B, M); return;
        case 32: fno_mix_wgrad_tc<32><<<M, 128, mix_wgrad_tc_smem(32), f->st>>>(X, dY, gw, B, M); return;
        default: break;
    }
    fno_mix_wgrad<<<M, 256, sizeof(float2) * 2 * 16 * C, f->st>>>(X, dY, gw, B, C, M);
}

// ---- forward / backward enqueue ------------------------------------------
void enqueue_forward(sp_fno* f, const float* x, long long x_bs, const float* cond, int B,
                     float* out) {
    const sp_fno_shape& s = f->s;
    const FnoOffsets& o = f->off;
    const int C = s.width, H = s.hidden, L = s.layers, G = f->G;
    const long long stride_h = fieldC(f);            // buffers are sized for max_batch
    const long long stride_X = (long long)s.max_batch * C * f->M;
    // conditioning MLP
    fno_dense<<<(B * H + 127) / 128, 128, 0, f->st>>>(cond, s.cond, f->pb + o.film1_w,
                                                      f->pb + o.film1_b, H, B, 1, f->hid_pre, f->hid);
    fno_dense<<<(B * G + 127) / 128, 128, 0, f->st>>>(f->hid, H, f->pb + o.film2_w,
                                                      f->pb + o.film2_b, G, B, 0, nullptr, f->g);
    // lift
    PW a = pw_base(f, B);
    a.in = x; a.in_bs = x_bs; a.cin = s.in_ch; a.cout = C;
    a.w = f->pb + o.lift_w; a.bias = f->pb + o.lift_b; a.out = f->h;
    pointwise(f, a);
    for (int k = 0; k < L; k++) {
        float* hk = f->h + k * stride_h;
        float2* Xk = f->X + k * stride_X;
        analysis(f, hk, Xk, B * C, f->s_one);
        mix(f, Xk, f->pb + o.spec[k], f->Y, B, 0);
        synthesis(f, f->Y, f->sbuf, B * C, f->s_inv, 0);
        PW l = pw_base(f, B);
        l.in = hk; l.in_bs = (long long)C * f->P; l.cin = C; l.cout = C;
        l.w = f->pb + o.lin_w[k]; l.bias = f->pb + o.lin_b[k];
        l.add = f->sbuf; l.film = f->g + 2 * k * C; l.fs = G; l.act = 1;
        l.pre = f->u + k * stride_h; l.out = f->h + (k + 1) * stride_h;
        pointwise(f, l);
    }
    PW p1 = pw_base(f, B);
    p1.in = f->h + L * stride_h; p1.in_bs = (long long)C * f->P; p1.cin = C; p1.cout = H;
    p1.w = f->pb + o.proj1_w; p1.bias = f->pb + o.proj1_b; p1.act = 1; p1.pre = f->q; p1.out = f->a;
    pointwise(f, p1);
    PW p2 = pw_base(f, B);
    p2.in = f->a; p2.in_bs = (long long)H * f->P; p2.cin = H; p2.cout = s.out_ch;
    p2.w = f->pb + o.proj2_w; p2.bias = f->pb + o.proj2_b; p2.out = out;
    pointwise(f, p2);
    f->last_x = x;
    f->last_x_bs = x_bs;
    f->last_cond = cond;
    f->last_out = out;
    f->last_batch = B;
}

void enqueue_backward(sp_fno* f, const float* target, int B) {
    const sp_fno_shape& s = f->s;
    const FnoOffsets& o = f->off;
    const int C = s.width, H = s.hidden, L = s.layers, G = f->G, P = f->P;
    const long long stride_h = fieldC(f);
    const long long stride_X = (long long)s.max_batch * C * f->M;
    const long long N = (long long)B * s.out_ch * P;
    fno_mse<<<kLossBlocks, 256, 0, f->st>>>(f->last_out, target, N, 2.0f / (float)N, f->dout,
                                            f->loss_part);
    fno_mse_final<<<1, 256, 0, f->st>>>(f->loss_part, kLossBlocks, 1.0f / (float)N, f->loss);
    // projection
    wgrad(f, f->dout, f->a, (long long)H * P, s.out_ch, H, B, f->grad + o.proj2_w,
          f->grad + o.proj2_b);
    PW t2 = pw_base(f, B);
    t2.in = f->dout; t2.in_bs = (long long)s.out_ch * P; t2.cin = s.out_ch; t2.cout = H;
    t2.w = f->pb + o.proj2_w; t2.trans = 1; t2.act = 2; t2.gate = f->q; t2.out = f->dq;
    pointwise(f, t2);
    const float* hL = f->h + L * stride_h;
    wgrad(f, f->dq, hL, (long long)C * P, H, C, B, f->grad + o.proj1_w, f->grad + o.proj1_b);
    PW t1 = pw_base(f, B);
    t1.in = f->dq; t1.in_bs = (long long)H * P; t1.cin = H; t1.cout = C;
    t1.w = f->pb + o.proj1_w; t1.trans = 1; t1.out = f->dhA;
    pointwise(f, t1);
    // layers, last to first
    float* dh = f->dhA;
    float* dh_next = f->dhB;
    for (int k = L - 1; k >= 0; k--) {
        const float* hk = f->h + k * stride_h;
        const float2* Xk = f->X + k * stride_X;
        fno_film_back<<<B * C, 256, 0, f->st>>>(dh, f->u + k * stride_h, f->g, C, P, G, k, f->du,
                                                f->dg);
        wgrad(f, f->du, hk, (long long)C * P, C, C, B, f->grad + o.lin_w[k], f->grad + o.lin_b[k]);
        PW tl = pw_base(f, B);
        tl.in = f->du; tl.in_bs = (long long)C * P; tl.cin = C; tl.cout = C;
        tl.w = f->pb + o.lin_w[k]; tl.trans = 1; tl.out = dh_next;
        pointwise(f, tl);
        analysis(f, f->du, f->dY, B * C, f->s_inv);
        mix_wgrad(f, Xk, f->dY, f->grad + o.spec[k], B);
        mix(f, f->dY, f->pb + o.spec[k], f->dX, B, 1);
        synthesis(f, f->dX, dh_next, B * C, f->s_one, 1);
        float* t = dh;
        dh = dh_next;
        dh_next = t;
    }
    // lift
    wgrad(f, dh, f->last_x, f->last_x_bs, C, s.in_ch, B, f->grad + o.lift_w, f->grad + o.lift_b);
    // conditioning MLP
    const int E2 = G * H + G;
    fno_dense_wgrad<<<(E2 + 127) / 128, 128, 0, f->st>>>(f->dg, f->hid, B, G, H,
                                                         f->grad + o.film2_w, f->grad + o.film2_b);
    fno_dense_dinput<<<(B * H + 127) / 128, 128, 0, f->st>>>(f->dg, f->pb + o.film2_w, B, G, H,
                                                             f->hid_pre, f->dhid);
    const int E1 = H * s.cond + H;
    fno_dense_wgrad<<<(E1 + 127) / 128, 128, 0, f->st>>>(f->dhid, f->last_cond, B, H, s.cond,
                                                         f->grad + o.film1_w, f->grad + o.film1_b);
}

void enqueue_adam(sp_fno* f) {
    const long long n = f->off.total;
    const int nb = (int)std::min<long long>((n + 255) / 256, 4096);
    fno_adam<<<nb, 256, 0, f->st>>>(f->p, f->pb, f->grad, f->am, f->av, n, f->hyper);
}

// host half of an Adam step: bias corrections for the next step count
void adam_hyper(sp_fno* f, float lr, float b1, float b2, float eps) {
    f->adam_t++;
    const double t = (double)f->adam_t;
    f->hyper_h[0] = (float)((double)lr / (1.0 - std::pow((double)b1, t)));
    f->hyper_h[1] = (float)std::sqrt(1.0 - std::pow((double)b2, t));
    f->hyper_h[2] = b1;
    f->hyper_h[3] = b2;
    f->hyper_h[4] = eps;
}

// the caller's stream -> the handle's stream, and back after the work
int join_in(sp_fno* f, void* stream) {
    cudaError_t e = cudaEventRecord(f->ev_in, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(f->st, f->ev_in, 0);
    return e == cudaSuccess ? SP_OK : cuda_fail(f, e, "stream join");
}

int join_out(sp_fno* f, void* stream, const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(f, e, what);
    e = cudaEventRecord(f->ev_out, f->st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent((cudaStream_t)stream, f->ev_out, 0);
    return e == cudaSuccess ? SP_OK : cuda_fail(f, e, what);
}

int check_batch(sp_fno* f, int batch) {
    if (batch < 1 || batch > f->s.max_batch)
        return fail(f, SP_E_INVALID, "batch outside 1 .. max_batch");
    return SP_OK;
}

}  // namespace

extern "C" {

int sp_fno_create(const sp_fno_shape* shape, sp_fno** out) {
    if (!shape || !out) return SP_E_INVALID;
    *out = nullptr;
    const sp_fno_shape& s = *shape;
    if (s.n < 4 || s.n > 64 || s.modes < 1 || 2 * s.modes > s.n || s.width < 1 || s.width > 64 ||
        s.layers < 1 || s.layers > 8 || s.in_ch < 1 || s.in_ch > 16 || s.out_ch < 1 ||
        s.out_ch > 16 || s.cond < 1 || s.cond > 16 || s.hidden < 1 || s.hidden > 64 ||
        s.max_batch < 1 || s.max_batch > 1024)
        return SP_E_INVALID;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return SP_E_CUDA;    // no usable CUDA device
    }
    sp_fno* f = new sp_fno();
    f->s = s;
    f->off = offsets(s);
    f->P = s.n * s.n;
    f->M = 2 * s.modes * s.modes;
    f->G = 2 * s.layers * s.width;
    const long long np = f->off.total;
    const long long Bm = s.max_batch, C = s.width, H = s.hidden, P = f->P, M = f->M;
    bool ok = true;
    f->p = dalloc<float>(f, np, ok);
    f->grad = dalloc<float>(f, np, ok);
    f->am = dalloc<float>(f, np, ok);
    f->av = dalloc<float>(f, np, ok);
    f->pb = dalloc<uint16_t>(f, np, ok);
    f->hyper = dalloc<float>(f, 8, ok);
    f->tw = dalloc<float2>(f, s.n, ok);
    const DftTc DL = dft_tc_layout(s.n, s.modes);
    const bool dft_tc = dft_tc_ok(s.n, s.modes);
    if (dft_tc) {
        f->tA1 = dalloc<float>(f, (long long)s.n * DL.N2, ok);
        f->tA2 = dalloc<float>(f, (long long)DL.R4 * s.n, ok);
        f->tS1 = dalloc<float>(f, (long long)s.n * DL.R4, ok);
        f->tS2 = dalloc<float>(f, (long long)DL.K2 * s.n, ok);
    }
    f->s_one = dalloc<float>(f, s.modes, ok);
    f->s_inv = dalloc<float>(f, s.modes, ok);
    const long long FC = Bm * C * P;
    f->h = dalloc<float>(f, FC * (s.layers + 1), ok);
    f->u = dalloc<float>(f, FC * s.layers, ok);
    f->X = dalloc<float2>(f, Bm * C * M * s.layers, ok);
    f->Y = dalloc<float2>(f, Bm * C * M, ok);
    f->sbuf = dalloc<float>(f, FC, ok);
    f->q = dalloc<float>(f, Bm * H * P, ok);
    f->a = dalloc<float>(f, Bm * H * P, ok);
    f->g = dalloc<float>(f, Bm * f->G, ok);
    f->hid_pre = dalloc<float>(f, Bm * H, ok);
    f->hid = dalloc<float>(f, Bm * H, ok);
    f->out = dalloc<float>(f, Bm * s.out_ch * P, ok);
    f->dout = dalloc<float>(f, Bm * s.out_ch * P, ok);
    f->dq = dalloc<float>(f, Bm * H * P, ok);
    f->dhA = dalloc<float>(f, FC, ok);
    f->dhB = dalloc<float>(f, FC, ok);
    f->du = dalloc<float>(f, FC, ok);
    f->dY = dalloc<float2>(f, Bm * C * M, ok);
    f->dX = dalloc<float2>(f, Bm * C * M, ok);
    f->dg = dalloc<float>(f, Bm * f->G, ok);
    f->dhid = dalloc<float>(f, Bm * H, ok);
    const long long tiles = (P + kTile - 1) / kTile;
    const long long mo = std::max<long long>(std::max(C, H), s.out_ch);
    const long long mi = std::max<long long>(std::max(C, H), s.in_ch);
    f->part = dalloc<float>(f, Bm * tiles * (mo * mi + mo), ok);
    f->loss_part = dalloc<float>(f, kLossBlocks, ok);
    f->loss = dalloc<float>(f, 1, ok);
    f->cond_b = dalloc<float>(f, Bm * s.cond, ok);
    f->target_b = dalloc<float>(f, Bm * s.out_ch * P, ok);
    f->x_b = dalloc<float>(f, Bm * s.in_ch * P, ok);
    f->idx_d = dalloc<int>(f, Bm, ok);
    if (!ok) {
        sp_fno_destroy(f);
        return SP_E_NOMEM;
    }
    cudaError_t e = cudaStreamCreateWithFlags(&f->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f->ev_in, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f->ev_out, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocHost(&f->idx_h, sizeof(int32_t) * Bm);
    if (e == cudaSuccess) e = cudaMallocHost(&f->hyper_h, sizeof(float) * 8);
    if (e != cudaSuccess) {
        sp_fno_destroy(f);
        return SP_E_CUDA;
    }
    // the weight-gradient tiles of 64 x 64 channel pairs take 66 KB, the
    // tensor-core mode mix of width 64 70 KB
    e = cudaFuncSetAttribute(fno_wgrad_partial_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(float) * 128 * kLdTc));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(fno_mix_tc<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)mix_tc_smem(64));
    if (e != cudaSuccess) {
        sp_fno_destroy(f);
        return SP_E_CUDA;
    }
    // twiddles and per-ky scales from double precision
    std::vector<float2> tw(s.n);
    for (int k = 0; k < s.n; k++) {
        const double th = 6.283185307179586477 * (double)k / (double)s.n;
        tw[k] = make_float2((float)std::cos(th), (float)std::sin(th));
    }
    std::vector<float> one(s.modes, 1.0f), inv(s.modes);
    for (int k = 0; k < s.modes; k++)
        inv[k] = (float)((k == 0 ? 1.0 : 2.0) / ((double)s.n * (double)s.n));
    e = cudaMemcpy(f->tw, tw.data(), sizeof(float2) * s.n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && dft_tc) {
        // the DFT matrices of the tensor-core kernels, from double precision
        const int n = s.n, m = s.modes, N2 = DL.N2, K2 = DL.K2, R4 = DL.R4;
        auto cs = [n](long long k, bool sine) {
            const double th = 6.283185307179586477 * (double)(((k % n) + n) % n) / (double)n;
            return (float)(sine ? std::sin(th) : std::cos(th));
        };
        auto kx_of = [n, m](int kxi) { return kxi < m ? kxi : n - 2 * m + kxi; };
        std::vector<float> a1((size_t)n * N2, 0.0f), a2((size_t)R4 * n, 0.0f);
        std::vector<float> s1((size_t)n * R4), s2((size_t)K2 * n, 0.0f);
        for (int y = 0; y < n; y++)
            for (int c = 0; c < 2 * m; c++)
                a1[(size_t)y * N2 + c] = c < m ? cs((long long)c * y, false)
                                               : -cs((long long)(c - m) * y, true);
        for (int r = 0; r < 4 * m; r++)
            for (int x = 0; x < n; x++)
                a2[(size_t)r * n + x] = r < 2 * m ? cs((long long)kx_of(r) * x, false)
                                                  : cs((long long)kx_of(r - 2 * m) * x, true);
        for (int x = 0; x < n; x++)
            for (int k = 0; k < R4; k++) s1[(size_t)x * R4 + k] = a2[(size_t)k * n + x];
        for (int c = 0; c < N2; c++)
            for (int y = 0; y < n; y++) s2[(size_t)c * n + y] = a1[(size_t)y * N2 + c];
        e = cudaMemcpy(f->tA1, a1.data(), sizeof(float) * a1.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(f->tA2, a2.data(), sizeof(float) * a2.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(f->tS1, s1.data(), sizeof(float) * s1.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(f->tS2, s2.data(), sizeof(float) * s2.size(), cudaMemcpyHostToDevice);
        // the attribute is per kernel, not per network: the largest shape
        // of the tensor-core path (n = 64, 2m = 32), so that networks of
        // several shapes can share a process
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(fno_analysis_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)dft_tc_smem(64, 16, false));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(fno_synthesis_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)dft_tc_smem(64, 16, true));
    }
    if (e == cudaSuccess)
        e = cudaMemcpy(f->s_one, one.data(), sizeof(float) * s.modes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(f->s_inv, inv.data(), sizeof(float) * s.modes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(f->p, 0, sizeof(float) * np);
    if (e == cudaSuccess) e = cudaMemset(f->pb, 0, sizeof(uint16_t) * np);
    if (e == cudaSuccess) e = cudaMemset(f->grad, 0, sizeof(float) * np);
    if (e == cudaSuccess) e = cudaMemset(f->am, 0, sizeof(float) * np);
    if (e == cudaSuccess) e = cudaMemset(f->av, 0, sizeof(float) * np);
    if (e != cudaSuccess) {
        sp_fno_destroy(f);
        return SP_E_CUDA;
    }
    *out = f;
    return SP_OK;
}

int64_t sp_fno_num_params(const sp_fno* f) { return f ? f->off.total : -1; }

int sp_fno_set_params(sp_fno* f, const float* params, int64_t count) {
    if (!f) return SP_E_INVALID;
    if (!params || count != f->off.total) return fail(f, SP_E_INVALID, "parameter count mismatch");
    const long long n = f->off.total;
    cudaError_t e = cudaMemcpy(f->p, params, sizeof(float) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemsetAsync(f->am, 0, sizeof(float) * n, f->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(f->av, 0, sizeof(float) * n, f->st);
    if (e != cudaSuccess) return cuda_fail(f, e, "sp_fno_set_params");
    fno_to_bf16<<<(int)std::min<long long>((n + 255) / 256, 4096), 256, 0, f->st>>>(f->p, f->pb, n);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->st);
    if (e != cudaSuccess) return cuda_fail(f, e, "sp_fno_set_params");
    f->adam_t = 0;
    return SP_OK;
}

int sp_fno_get_params(sp_fno* f, float* params, int64_t count) {
    if (!f) return SP_E_INVALID;
    if (!params || count != f->off.total) return fail(f, SP_E_INVALID, "parameter count mismatch");
    cudaError_t e = cudaStreamSynchronize(f->st);
    if (e == cudaSuccess)
        e = cudaMemcpy(params, f->p, sizeof(float) * count, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? SP_OK : cuda_fail(f, e, "sp_fno_get_params");
}

int sp_fno_get_grads(sp_fno* f, float* grads, int64_t count) {
    if (!f) return SP_E_INVALID;
    if (!grads || count != f->off.total) return fail(f, SP_E_INVALID, "parameter count mismatch");
    cudaError_t e = cudaStreamSynchronize(f->st);
    if (e == cudaSuccess)
        e = cudaMemcpy(grads, f->grad, sizeof(float) * count, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? SP_OK : cuda_fail(f, e, "sp_fno_get_grads");
}

int sp_fno_forward(sp_fno* f, const float* x, int32_t x_shared, const float* cond, int32_t batch,
                   float* out, void* stream) {
    if (!f) return SP_E_INVALID;
    if (!x || !cond || !out) return fail(f, SP_E_INVALID, "sp_fno_forward: null pointer");
    int rc = check_batch(f, batch);
    if (rc) return rc;
    if ((rc = join_in(f, stream))) return rc;
    enqueue_forward(f, x, x_shared ? 0 : (long long)f->s.in_ch * f->P, cond, batch, out);
    return join_out(f, stream, "sp_fno_forward");
}

int sp_fno_backward(sp_fno* f, const float* target, int32_t batch, void* stream) {
    if (!f) return SP_E_INVALID;
    if (!target) return fail(f, SP_E_INVALID, "sp_fno_backward: null target");
    int rc = check_batch(f, batch);
    if (rc) return rc;
    if (batch != f->last_batch || !f->last_out)
        return fail(f, SP_E_INVALID, "sp_fno_backward: no forward pass of this batch");
    if ((rc = join_in(f, stream))) return rc;
    enqueue_backward(f, target, batch);
    return join_out(f, stream, "sp_fno_backward");
}

int sp_fno_adam(sp_fno* f, float lr, float beta1, float beta2, float eps, void* stream) {
    if (!f) return SP_E_INVALID;
    int rc = join_in(f, stream);
    if (rc) return rc;
    adam_hyper(f, lr, beta1, beta2, eps);
    cudaError_t e = cudaMemcpyAsync(f->hyper, f->hyper_h, sizeof(float) * 5,
                                    cudaMemcpyHostToDevice, f->st);
    if (e != cudaSuccess) return cuda_fail(f, e, "sp_fno_adam");
    enqueue_adam(f);
    // the pinned staging is reused by the next call
    e = cudaStreamSynchronize(f->st);
    if (e != cudaSuccess) return cuda_fail(f, e, "sp_fno_adam");
    return join_out(f, stream, "sp_fno_adam");
}

int sp_fno_train_step(sp_fno* f, const float* x, int32_t x_shared, const float* cond,
                      const float* target, int32_t rows, const int32_t* idx, int32_t batch,
                      float lr, float beta1, float beta2, float eps, void* stream) {
    if (!f) return SP_E_INVALID;
    if (!x || !cond || !target || !idx)
        return fail(f, SP_E_INVALID, "sp_fno_train_step: null pointer");
    int rc = check_batch(f, batch);
    if (rc) return rc;
    for (int j = 0; j < batch; j++)
        if (idx[j] < 0 || idx[j] >= rows)
            return fail(f, SP_E_INVALID, "sp_fno_train_step: row index outside 0 .. rows-1");
    if ((rc = join_in(f, stream))) return rc;
    // the previous step's copies out of the pinned staging must be done
    cudaError_t e = cudaStreamSynchronize(f->st);
    if (e != cudaSuccess) return cuda_fail(f, e, "sp_fno_train_step");
    memcpy(f->idx_h, idx, sizeof(int32_t) * batch);
    adam_hyper(f, lr, beta1, beta2, eps);
    e = cudaMemcpyAsync(f->idx_d, f->idx_h, sizeof(int32_t) * batch, cudaMemcpyHostToDevice, f->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(f->hyper, f->hyper_h, sizeof(float) * 5, cudaMemcpyHostToDevice, f->st);
    if (e != cudaSuccess) return cuda_fail(f, e, "sp_fno_train_step");
    sp_fno::Graph* gr = nullptr;
    for (auto& c : f->graphs)
        if (c.x == x && c.cond == cond && c.target == target && c.x_shared == x_shared &&
            c.batch == batch)
            gr = &c;
    if (!gr) {
        sp_fno::Graph c;
        c.x = x; c.cond = cond; c.target = target; c.x_shared = x_shared; c.batch = batch;
        cudaGraph_t graph = nullptr;
        e = cudaStreamBeginCapture(f->st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_fail(f, e, "sp_fno_train_step: capture");
        const sp_fno_shape& s = f->s;
        const int gb = 1024;
        fno_gather<<<gb, 256, 0, f->st>>>(cond, f->idx_d, batch, s.cond, f->cond_b);
        fno_gather<<<gb, 256, 0, f->st>>>(target, f->idx_d, batch, (long long)s.out_ch * f->P,
                                          f->target_b);
        const float* xin = x;
        long long xbs = 0;
        if (!x_shared) {
            fno_gather<<<gb, 256, 0, f->st>>>(x, f->idx_d, batch, (long long)s.in_ch * f->P, f->x_b);
            xin = f->x_b;
            xbs = (long long)s.in_ch * f->P;
        }
        enqueue_forward(f, xin, xbs, f->cond_b, batch, f->out);
        enqueue_backward(f, f->target_b, batch);
        enqueue_adam(f);
        cudaError_t le = cudaGetLastError();
        e = cudaStreamEndCapture(f->st, &graph);
        if (le != cudaSuccess) e = le;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&c.exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) return cuda_fail(f, e, "sp_fno_train_step: graph");
        f->graphs.push_back(c);
        gr = &f->graphs.back();
    } else {
        // the forward state a later sp_fno_backward would read
        f->last_x = x_shared ? x : f->x_b;
        f->last_x_bs = x_shared ? 0 : (long long)f->s.in_ch * f->P;
        f->last_cond = f->cond_b;
        f->last_out = f->out;
        f->last_batch = batch;
    }
    e = cudaGraphLaunch(gr->exec, f->st);
    if (e != cudaSuccess) return cuda_fail(f, e, "sp_fno_train_step: launch");
    return join_out(f, stream, "sp_fno_train_step");
}

int sp_fno_loss(sp_fno* f, float* loss) {
    if (!f || !loss) return SP_E_INVALID;
    cudaError_t e = cudaStreamSynchronize(f->st);
    if (e == cudaSuccess) e = cudaMemcpy(loss, f->loss, sizeof(float), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? SP_OK : cuda_fail(f, e, "sp_fno_loss");
}

const char* sp_fno_last_error(sp_fno* f) { return f ? f->err.c_str() : "null handle"; }

void sp_fno_destroy(sp_fno* f) {
    if (!f) return;
    if (f->st) cudaStreamSynchronize(f->st);
    for (auto& c : f->graphs)
        if (c.exec) cudaGraphExecDestroy(c.exec);
    for (void* ptr : f->allocs) cudaFree(ptr);
    if (f->idx_h) cudaFreeHost(f->idx_h);
    if (f->hyper_h) cudaFreeHost(f->hyper_h);
    if (f->ev_in) cudaEventDestroy(f->ev_in);
    if (f->ev_out) cudaEventDestroy(f->ev_out);
    if (f->st) cudaStreamDestroy(f->st);
    delete f;
}

}  // extern "C"
