/*
 * sp_oracle.c — TEST INFRASTRUCTURE.  CPU restatement of the SpatialPy NSM
 * hot path (see sp_oracle.h).  Compiled with -ffp-contract=off so every
 * floating-point operation rounds exactly as written; the GPU engine uses the
 * same operation order and is compared with this file bit for bit.
 */
#include "sp_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ------------------------------------------------------------------------
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies with the
 * published multipliers and Weyl key increments.
 * ------------------------------------------------------------------------ */
void spo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* u in (0,1) from 32 random bits: (r + 1/2) 2^-32, exact in double */
static inline double u01(uint32_t r) { return ((double)r + 0.5) * (1.0 / 4294967296.0); }

/* ------------------------------------------------------------------------
 * -log(u), u in (0,1).  Cody-Waite style reduction u = m 2^e with m in
 * [sqrt(1/2), sqrt(2)), then log m = 2 atanh(z), z = (m-1)/(m+1), summed as
 * the Maclaurin series of atanh (coefficients 1/(2k+1)) to w^10, w = z^2,
 * |z| <= 0.1716 so the truncation error is below 1e-18.  ln 2 is split into
 * a head with the low 21 mantissa bits cleared (e * head is exact for
 * |e| < 2^21) and the double nearest to ln 2 - head.
 * ------------------------------------------------------------------------ */
double spo_neglog(double u) {
    uint64_t b;
    memcpy(&b, &u, 8);
    int e = (int)((b >> 52) & 0x7ff) - 1023;
    b = (b & 0x000fffffffffffffull) | 0x3ff0000000000000ull;   /* m in [1,2) */
    double m;
    memcpy(&m, &b, 8);
    if (m > 1.4142135623730951) { m = m * 0.5; e = e + 1; }
    double z = (m - 1.0) / (m + 1.0);
    double w = z * z;
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
    double logm = (2.0 * z) * p;
    const double ln2_hi = 6.931471803691238e-01;    /* 0x3fe62e42fee00000 */
    const double ln2_lo = 1.9082149292705877e-10;   /* 0x3dea39ef35793c76 */
    double ed = (double)e;
    double r = ed * ln2_hi + (ed * ln2_lo + logm);
    return -r;
}

/* ------------------------------------------------------------------------
 * Single-precision variate helpers used by the NSM event loop.
 *   u24(r):  (r >> 8) 2^-24 + 2^-25, exact, in (0,1)      (selection uniforms)
 *   u32f(r): ((float)r + 0.5f) 2^-32, in (0,1]              (exponential draws)
 *   neglog_f: the construction of spo_neglog in float, series to w^5 and a
 *   ln 2 head with the low 9 mantissa bits cleared.
 * ------------------------------------------------------------------------ */
static inline float u24(uint32_t r) {
    return (float)(r >> 8) * (1.0f / 16777216.0f) + (1.0f / 33554432.0f);
}
static inline float u32f(uint32_t r) { return ((float)r + 0.5f) * (1.0f / 4294967296.0f); }

float spo_neglog_f(float u) {
    uint32_t b;
    memcpy(&b, &u, 4);
    int e = (int)((b >> 23) & 0xff) - 127;
    b = (b & 0x007fffffu) | 0x3f800000u;
    float m;
    memcpy(&m, &b, 4);
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
    const float ln2_hi = 0.693145751953125f;     /* 0x3f317200 */
    const float ln2_lo = 1.428606765330187e-06f; /* 0x35bfbe8e */
    const float ed = (float)e;
    return -(ed * ln2_hi + (ed * ln2_lo + logm));
}

/* ------------------------------------------------------------------------
 * Neighbour search with the ANN fixed-radius predicate.
 * ------------------------------------------------------------------------ */
typedef struct { double d2; int32_t j; } cand_t;

static int cand_less(const cand_t *a, const cand_t *b) {
    return a->d2 < b->d2 || (a->d2 == b->d2 && a->j < b->j);
}

static double kernel_alpha(int dim, double h) {
    /* particle.cpp:168-175 (1D: `5 / 4 * h` is integer 5/4 = 1 times h) */
    if (dim == 3) return 105 / (16 * M_PI * h * h * h);
    if (dim == 2) return 5 / (M_PI * h * h);
    return 1 * h;
}

int spo_neighbors(int32_t n, int32_t dim, const double *xq, const double *xt, double h,
                  const double *mass, const double *rho, int32_t kmax, int32_t *count,
                  int32_t *idx, double *dist, double *dwdr, double *dij) {
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int d = 0; d < dim; d++) {
        lo[d] = hi[d] = xt[d];
        for (int i = 0; i < n; i++) {
            double a = xt[3 * i + d], b = xq[3 * i + d];
            if (a < lo[d]) lo[d] = a;
            if (b < lo[d]) lo[d] = b;
            if (a > hi[d]) hi[d] = a;
            if (b > hi[d]) hi[d] = b;
        }
    }
    const double cs = h * 1.0000001;
    int nc[3] = {1, 1, 1};
    for (int d = 0; d < dim; d++) nc[d] = (int)floor((hi[d] - lo[d]) / cs) + 1;
    const long ncell = (long)nc[0] * nc[1] * nc[2];
    int32_t *start = (int32_t *)calloc((size_t)ncell + 1, sizeof(int32_t));
    int32_t *cell = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int32_t *order = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    #define CELLC(p, d) ((d) < dim ? (int)fmin(nc[d] - 1, floor(((p) - lo[d]) / cs)) : 0)
    for (int i = 0; i < n; i++) {
        int c0 = CELLC(xt[3 * i], 0), c1 = CELLC(xt[3 * i + 1], 1), c2 = CELLC(xt[3 * i + 2], 2);
        cell[i] = (int32_t)(((long)c0 * nc[1] + c1) * nc[2] + c2);
        start[cell[i] + 1]++;
    }
    for (long c = 0; c < ncell; c++) start[c + 1] += start[c];
    int32_t *fill = (int32_t *)malloc(sizeof(int32_t) * (size_t)ncell);
    memcpy(fill, start, sizeof(int32_t) * (size_t)ncell);
    for (int i = 0; i < n; i++) order[fill[cell[i]]++] = i;
    free(fill);

    const double sq = h * h;          /* ANNdist dist = system->h * system->h (particle.cpp:253) */
    const double alpha = kernel_alpha(dim, h);
    int rc = 0;
    cand_t *cand = (cand_t *)malloc(sizeof(cand_t) * (size_t)(kmax + 1));
    for (int i = 0; i < n && rc == 0; i++) {
        const double *q = xq + 3 * i;
        int qc[3];
        for (int d = 0; d < 3; d++) qc[d] = CELLC(q[d], d);
        int m = 0;
        for (int a = qc[0] - 1; a <= qc[0] + 1; a++) {
            if (a < 0 || a >= nc[0]) continue;
            for (int b = qc[1] - 1; b <= qc[1] + 1; b++) {
                if (b < 0 || b >= nc[1]) continue;
                for (int c = qc[2] - 1; c <= qc[2] + 1; c++) {
                    if (c < 0 || c >= nc[2]) continue;
                    long cid = ((long)a * nc[1] + b) * nc[2] + c;
                    for (int32_t t = start[cid]; t < start[cid + 1]; t++) {
                        int j = order[t];
                        const double *p = xt + 3 * j;
                        double d2 = 0;
                        int d;
                        for (d = 0; d < dim; d++) {       /* kd_fix_rad_search.cpp:160-170 */
                            double tt = q[d] - p[d];
                            d2 = d2 + tt * tt;
                            if (d2 > sq) break;
                        }
                        if (d < dim || d2 == 0) continue;  /* :173-174, no self match */
                        if (sqrt(d2) > h) continue;         /* particle.cpp:160-162 */
                        if (m >= kmax) { rc = -1; break; }
                        cand_t cd = {d2, j};
                        int k = m++;
                        while (k > 0 && cand_less(&cd, &cand[k - 1])) { cand[k] = cand[k - 1]; k--; }
                        cand[k] = cd;
                    }
                    if (rc) break;
                }
                if (rc) break;
            }
            if (rc) break;
        }
        count[i] = m;
        for (int k = 0; k < m; k++) {
            const int j = cand[k].j;
            const double r2 = cand[k].d2;
            const double r = sqrt(r2);
            /* particle.cpp:165-187 */
            const double R = r / h;
            const double dW = alpha * (-12 * r / (h * h)) * ((1 - R) * (1 - R));
            const double ih = 1.0 / h;
            const double ihsq = ih * ih;
            const double dhr = h - r;
            const double wfd = -25.066903536973515383e0 * dhr * dhr * ihsq * ihsq * ihsq * ih;
            const double D = -2.0 * (mass[i] * mass[j]) / (mass[i] + mass[j]) * (rho[i] + rho[j]) /
                             (rho[i] * rho[j]) * r2 * wfd / (r2 + 0.01 * h * h);
            idx[(size_t)i * kmax + k] = j;
            if (dist) dist[(size_t)i * kmax + k] = r;
            if (dwdr) dwdr[(size_t)i * kmax + k] = dW;
            if (dij) dij[(size_t)i * kmax + k] = D;
        }
    }
    #undef CELLC
    free(cand);
    free(start);
    free(cell);
    free(order);
    return rc;
}

void spo_diffusion_tables(const sp_scenario *sc, int32_t kmax, const int32_t *count,
                          const int32_t *idx, const double *dij, float *ddiag, float *cdf) {
    /* Ddiag[s] = sum_k D(s,type_j) D_ij in list order (simulate_rdme.cpp:142-148),
       accumulated in double and rounded to float; cdf holds the rounded
       running sums scanned by the destination choice (:359-367). */
    const int S = sc->num_species, T = sc->num_types;
    for (int i = 0; i < sc->num_particles; i++) {
        for (int s = 0; s < S; s++) {
            double acc = 0.0;
            for (int k = 0; k < count[i]; k++) {
                const int j = idx[(size_t)i * kmax + k];
                const double dc = sc->diffusion[s * T + (sc->type[j] - 1)];
                acc = acc + dc * dij[(size_t)i * kmax + k];
                if (cdf) cdf[((size_t)i * S + s) * kmax + k] = (float)acc;
            }
            ddiag[(size_t)i * S + s] = (float)acc;
        }
    }
}

/* ------------------------------------------------------------------------
 * NSM.  Propensities, selection scans and exponential variates in single
 * precision; event times (the clock) in double.
 * ------------------------------------------------------------------------ */
typedef struct {
    const sp_scenario *sc;
    int N, S, R, T, K;
    int32_t *cnt, *idx;
    float *cdf, *ddiag, *vol, *ivol, *rate;
} nsm_tables_t;

static int tables_build(const sp_scenario *sc, nsm_tables_t *t) {
    const int N = sc->num_particles;
    memset(t, 0, sizeof(*t));
    t->sc = sc;
    t->N = N;
    t->S = sc->num_species;
    t->R = sc->num_reactions;
    t->T = sc->num_types;
    int K = 16;
    for (;;) {
        t->cnt = (int32_t *)malloc(sizeof(int32_t) * N);
        t->idx = (int32_t *)malloc(sizeof(int32_t) * (size_t)N * K);
        double *dij = (double *)malloc(sizeof(double) * (size_t)N * K);
        int rc = spo_neighbors(N, sc->dimension, sc->x, sc->x, sc->h, sc->mass, sc->rho, K,
                               t->cnt, t->idx, NULL, NULL, dij);
        if (rc == 0) {
            t->K = K;
            t->cdf = (float *)malloc(sizeof(float) * (size_t)N * t->S * K);
            t->ddiag = (float *)malloc(sizeof(float) * (size_t)N * t->S);
            spo_diffusion_tables(sc, K, t->cnt, t->idx, dij, t->ddiag, t->cdf);
            free(dij);
            break;
        }
        free(t->cnt);
        free(t->idx);
        free(dij);
        K *= 2;
    }
    t->vol = (float *)malloc(sizeof(float) * N);
    t->ivol = (float *)malloc(sizeof(float) * N);
    for (int i = 0; i < N; i++) {
        t->vol[i] = (float)(sc->mass[i] / sc->rho[i]);
        t->ivol[i] = (float)(sc->rho[i] / sc->mass[i]);
    }
    t->rate = (float *)malloc(sizeof(float) * (t->R > 0 ? t->R : 1));
    for (int r = 0; r < t->R; r++) t->rate[r] = (float)sc->rxn_rate[r];
    return 0;
}

static void tables_free(nsm_tables_t *t) {
    free(t->cnt); free(t->idx); free(t->cdf); free(t->ddiag); free(t->vol); free(t->ivol);
    free(t->rate);
}

/* a custom propensity program (SP_OP_* in spgpu.h) in double: the same
   operations in the same order as the kernels' interpreter (nsm_prog.cuh);
   the engine has checked the program before this runs */
static double run_program_x(const sp_scenario *sc, const int32_t *code, const double *consts,
                            const int32_t *xi, const double *xd, double vol, double tm, int type,
                            int v);

static double run_program(const sp_scenario *sc, int r, const int32_t *x, double vol, double tm,
                          int type, int v) {
    return run_program_x(sc, sc->rxn_code + sc->rxn_code_off[r], sc->rxn_consts, x, NULL, vol,
                         tm, type, v);
}

/* xi: integer counts, or xd: concentrations (exactly one is set) */
static double run_program_x(const sp_scenario *sc, const int32_t *code, const double *consts,
                            const int32_t *xi, const double *xd, double vol, double tm, int type,
                            int v) {
    double st[SP_PROG_MAX_STACK];
    int sp = 0;
    for (int pc = 0;;) {
        const int op = code[pc];
        if (op == SP_OP_END) return st[sp - 1];
        switch (op) {
            case SP_OP_CONST: st[sp++] = consts[code[pc + 1]]; pc += 2; continue;
            case SP_OP_X:
                st[sp++] = xd ? xd[code[pc + 1]] : (double)xi[code[pc + 1]];
                pc += 2;
                continue;
            case SP_OP_VOL: st[sp++] = vol; pc++; continue;
            case SP_OP_T: st[sp++] = tm; pc++; continue;
            case SP_OP_TYPE: st[sp++] = (double)type; pc++; continue;
            case SP_OP_DATA:
                st[sp++] = sc->data_fn[(size_t)code[pc + 1] * sc->num_particles + v];
                pc += 2;
                continue;
            case SP_OP_NEG: st[sp - 1] = -st[sp - 1]; pc++; continue;
            case SP_OP_NOT: st[sp - 1] = st[sp - 1] == 0.0 ? 1.0 : 0.0; pc++; continue;
            case SP_OP_POWI: {
                const int n = code[pc + 1], m = n < 0 ? -n : n;
                double p = 1.0;
                for (int q = 0; q < m; q++) p = p * st[sp - 1];
                st[sp - 1] = n < 0 ? 1.0 / p : p;
                pc += 2;
                continue;
            }
            case SP_OP_EXP: st[sp - 1] = exp(st[sp - 1]); pc++; continue;
            case SP_OP_EXP + 1: st[sp - 1] = log(st[sp - 1]); pc++; continue;
            case SP_OP_EXP + 2: st[sp - 1] = sqrt(st[sp - 1]); pc++; continue;
            case SP_OP_EXP + 3: st[sp - 1] = sin(st[sp - 1]); pc++; continue;
            case SP_OP_EXP + 4: st[sp - 1] = cos(st[sp - 1]); pc++; continue;
            case SP_OP_EXP + 5: st[sp - 1] = tan(st[sp - 1]); pc++; continue;
            case SP_OP_EXP + 6: st[sp - 1] = fabs(st[sp - 1]); pc++; continue;
            case SP_OP_EXP + 7: st[sp - 1] = log10(st[sp - 1]); pc++; continue;
            case SP_OP_EXP + 8: st[sp - 1] = floor(st[sp - 1]); pc++; continue;
            case SP_OP_CEIL: st[sp - 1] = ceil(st[sp - 1]); pc++; continue;
            default: break;
        }
        const double b = st[sp - 1], a = st[sp - 2];
        double res;
        switch (op) {
            case SP_OP_ADD: res = a + b; break;
            case SP_OP_SUB: res = a - b; break;
            case SP_OP_MUL: res = a * b; break;
            case SP_OP_DIV: res = a / b; break;
            case SP_OP_POW: res = pow(a, b); break;
            case SP_OP_LT: res = a < b ? 1.0 : 0.0; break;
            case SP_OP_LT + 1: res = a <= b ? 1.0 : 0.0; break;
            case SP_OP_LT + 2: res = a > b ? 1.0 : 0.0; break;
            case SP_OP_LT + 3: res = a >= b ? 1.0 : 0.0; break;
            case SP_OP_LT + 4: res = a == b ? 1.0 : 0.0; break;
            case SP_OP_NE: res = a != b ? 1.0 : 0.0; break;
            case SP_OP_AND: res = (a != 0.0 && b != 0.0) ? 1.0 : 0.0; break;
            default: res = (a != 0.0 || b != 0.0) ? 1.0 : 0.0; break;
        }
        st[sp - 2] = res;
        sp--;
        pc++;
    }
}

/* mass-action propensity in float, the generated code's operator order with
   the second-order division by vol replaced by a product with 1/vol
   (rounded from double): k*vol, k*A, (k*A*B)*(1/vol), (k*A*(A-1))*(1/vol);
   a custom propensity is its program's value at time tm, rounded to float */
static inline float prop(const nsm_tables_t *t, int r, const int32_t *x, float vol, float ivol,
                         int type, int v, double tm) {
    const sp_scenario *sc = t->sc;
    if (sc->rxn_allowed && !sc->rxn_allowed[(size_t)r * (sc->num_types + 1) + type]) return 0.0f;
    if (sc->rxn_kind[r] == SP_RXN_CUSTOM) return (float)run_program(sc, r, x, (double)vol, tm, type, v);
    const float k = t->rate[r];
    const int a = sc->rxn_reactants[2 * r], b = sc->rxn_reactants[2 * r + 1];
    switch (sc->rxn_kind[r]) {
        case SP_RXN_ZERO: return k * vol;
        case SP_RXN_FIRST: return k * (float)x[a];
        case SP_RXN_SECOND: return k * (float)x[a] * (float)x[b] * ivol;
        default: return k * (float)x[a] * (float)(x[a] - 1) * ivol;
    }
}

/* the voxel whose volume a rate uses: its own, or (reference selection, for
   a diffusion destination) the source voxel's; tm: the time custom
   propensities see */
static inline void voxel_rates(const nsm_tables_t *t, int v, const int32_t *x, int volv,
                               float *srr, float *sdr, double tm) {
    const float vol = t->vol[volv], ivol = t->ivol[volv];
    float a = 0.0f;
    for (int r = 0; r < t->R; r++) a = a + prop(t, r, x, vol, ivol, t->sc->type[v], v, tm);
    float d = 0.0f;
    for (int s = 0; s < t->S; s++) d = d + t->ddiag[(size_t)v * t->S + s] * (float)x[s];
    *srr = a;
    *sdr = d;
}

/* indexed binary heap over (tau, voxel) */
typedef struct { int n; int32_t *heap, *pos; double *tau; } heap_t;

static inline int hless(const heap_t *h, int a, int b) {
    return h->tau[a] < h->tau[b] || (h->tau[a] == h->tau[b] && a < b);
}
static void hswap(heap_t *h, int i, int j) {
    int32_t a = h->heap[i], b = h->heap[j];
    h->heap[i] = b; h->heap[j] = a;
    h->pos[b] = i; h->pos[a] = j;
}
static void hfix(heap_t *h, int v) {
    int i = h->pos[v];
    while (i > 0) {
        int p = (i - 1) / 2;
        if (!hless(h, h->heap[i], h->heap[p])) break;
        hswap(h, i, p);
        i = p;
    }
    for (;;) {
        int l = 2 * i + 1, r = l + 1, m = i;
        if (l < h->n && hless(h, h->heap[l], h->heap[m])) m = l;
        if (r < h->n && hless(h, h->heap[r], h->heap[m])) m = r;
        if (m == i) break;
        hswap(h, i, m);
        i = m;
    }
}

/* next firing time t + E/a (NRMConstant_v5.cpp:57, :98): the waiting time in
   float, the clock in double */
static inline double draw_time(double t, float e, float a) {
    return a > 0.0f ? t + (double)(e / a) : HUGE_VAL;
}

/* one trajectory's state between windows */
typedef struct {
    int32_t *x;
    heap_t h;
    uint32_t key[2];
    uint64_t evn;
    int64_t nrx, ndf;
    int status;
} nsm_state_t;

static void nsm_state_init(nsm_state_t *st, const nsm_tables_t *t, const uint32_t *u0,
                           uint64_t seed) {
    const int N = t->N, S = t->S;
    st->x = (int32_t *)malloc(sizeof(int32_t) * (size_t)N * S);
    for (size_t i = 0; i < (size_t)N * S; i++) st->x[i] = (int32_t)u0[i];
    st->h.n = N;
    st->h.heap = (int32_t *)malloc(sizeof(int32_t) * N);
    st->h.pos = (int32_t *)malloc(sizeof(int32_t) * N);
    st->h.tau = (double *)malloc(sizeof(double) * N);
    st->key[0] = (uint32_t)seed;
    st->key[1] = (uint32_t)(seed >> 32);
    st->evn = 0;
    st->nrx = st->ndf = 0;
    st->status = SP_TRAJ_OK;
}

static void nsm_state_free(nsm_state_t *st) {
    free(st->x); free(st->h.heap); free(st->h.pos); free(st->h.tau);
}

/* queue build at t0 (NRMConstant_v5::build, :52-71): Philox stream 1, counter
   (voxel, build_index) */
static void nsm_build(const nsm_tables_t *t, nsm_state_t *st, double t0, uint32_t build_index) {
    const int N = t->N, S = t->S;
    heap_t *h = &st->h;
    for (int v = 0; v < N; v++) {
        float srr, sdr;
        voxel_rates(t, v, st->x + (size_t)v * S, v, &srr, &sdr, 0.0);
        uint32_t ctr[4] = {(uint32_t)v, build_index, 1u, 0u}, r[4];
        spo_philox4x32_10(ctr, st->key, r);
        h->tau[v] = draw_time(t0, spo_neglog_f(u32f(r[0])), srr + sdr);
        h->heap[v] = v;
        h->pos[v] = v;
    }
    for (int i = N / 2 - 1; i >= 0; i--) {      /* heapify */
        int j = i;
        for (;;) {
            int l = 2 * j + 1, rr = l + 1, m = j;
            if (l < N && hless(h, h->heap[l], h->heap[m])) m = l;
            if (rr < N && hless(h, h->heap[rr], h->heap[m])) m = rr;
            if (m == j) break;
            hswap(h, j, m);
            j = m;
        }
    }
}

/* the events of one engine step, up to t_end = dt*step + dt
   (nsm_core__take_step, simulate_rdme.cpp:211-472) */
static void nsm_window(const nsm_tables_t *t, nsm_state_t *st, int step, int selection) {
    const sp_scenario *sc = t->sc;
    const int S = t->S, K = t->K;
    int32_t *x = st->x;
    heap_t *hp = &st->h;
    const double t_end = sc->dt * (double)step + sc->dt;   /* simulate_rdme.cpp:67,215 */
    for (;;) {
        const int v = hp->heap[0];
        const double tt = hp->tau[v];
        if (tt == HUGE_VAL) break;
        if (selection == SP_SELECT_EXACT && tt > t_end) break;
        uint32_t ctr[4] = {(uint32_t)st->evn, (uint32_t)(st->evn >> 32), 0u, 0u}, r[4];
        spo_philox4x32_10(ctr, st->key, r);
        st->evn++;
        const float ua = u24(r[0]), ub = u24(r[1]);
        const float e0 = spo_neglog_f(u32f(r[2])), e1 = spo_neglog_f(u32f(r[3]));
        int32_t *xv = x + (size_t)v * S;
        float srr, sdr;
        voxel_rates(t, v, xv, v, &srr, &sdr, tt);
        const float tot = srr + sdr;
        if (ua * tot <= srr) {                               /* :255 rand1 <= srrate/totrate */
            const float target = selection == SP_SELECT_EXACT ? ua * tot : ua * srr;
            float cum = 0.0f;
            int re = -1, last = -1;
            for (int q = 0; q < t->R; q++) {
                const float a = prop(t, q, xv, t->vol[v], t->ivol[v], sc->type[v], v, tt);
                cum = cum + a;
                if (a > 0.0f) {
                    last = q;
                    if (target <= cum) { re = q; break; }
                }
            }
            if (re < 0) re = last;
            if (re < 0) { st->status = SP_TRAJ_SELECT_OVERFLOW; break; }
            for (int64_t i = sc->jcN[re]; i < sc->jcN[re + 1]; i++) {   /* :285-296 */
                xv[sc->irN[i]] += sc->prN[i];
                if (xv[sc->irN[i]] < 0) st->status = SP_TRAJ_NEG_COUNT;
            }
            if (st->status) break;
            voxel_rates(t, v, xv, v, &srr, &sdr, tt);
            hp->tau[v] = draw_time(tt, e0, srr + sdr);
            hfix(hp, v);
            st->nrx++;
        } else {
            const float target = selection == SP_SELECT_EXACT ? ua * tot - srr : ua * sdr;
            float cum = 0.0f;
            int sp = -1, last = -1;
            for (int s = 0; s < S; s++) {                      /* :319-321 */
                const float wgt = t->ddiag[(size_t)v * S + s] * (float)xv[s];
                cum = cum + wgt;
                if (wgt > 0.0f) {
                    last = s;
                    if (target <= cum) { sp = s; break; }
                }
            }
            if (sp < 0) sp = last;
            if (sp < 0) { st->status = SP_TRAJ_SELECT_OVERFLOW; break; }
            const float target2 = ub * t->ddiag[(size_t)v * S + sp];   /* :353-354 */
            const float *c = t->cdf + ((size_t)v * S + sp) * K;
            int k = -1, lastk = -1;
            float prev = 0.0f;
            for (int q = 0; q < t->cnt[v]; q++) {             /* :359-367 */
                if (c[q] > prev) {
                    lastk = q;
                    if (c[q] > target2) { k = q; break; }
                }
                prev = c[q];
            }
            if (k < 0) k = lastk;
            if (k < 0) { st->status = SP_TRAJ_SELECT_OVERFLOW; break; }
            const int w = t->idx[(size_t)v * K + k];
            int32_t *xw = x + (size_t)w * S;
            xv[sp] -= 1;                                          /* :394-402 */
            xw[sp] += 1;            /* w == v (a moving particle's own start-of-step
                                       point in its list): the count is unchanged */
            voxel_rates(t, v, xv, v, &srr, &sdr, tt);
            hp->tau[v] = draw_time(tt, e0, srr + sdr);
            hfix(hp, v);
            /* the engine evaluates the destination's reactions with the
               source voxel's volume (simulate_rdme.cpp:431-433) */
            voxel_rates(t, w, xw, selection == SP_SELECT_REFERENCE ? v : w, &srr, &sdr, tt);
            hp->tau[w] = draw_time(tt, e1, srr + sdr);
            hfix(hp, w);
            st->ndf++;
        }
        if (selection == SP_SELECT_REFERENCE && tt > t_end) break;   /* :233 */
    }
}

/* static domain: one queue build at t = 0, then every step's window */
static int nsm_run(const nsm_tables_t *t, const uint32_t *u0, uint64_t seed, int selection,
                   int32_t *out, int64_t *ev) {
    const sp_scenario *sc = t->sc;
    const size_t NS = (size_t)t->N * t->S;
    nsm_state_t st;
    nsm_state_init(&st, t, u0, seed);
    nsm_build(t, &st, 0.0, 0u);
    int oi = 0;
    const int nout = sc->num_outputs;
    for (int step = 0; step < sc->num_steps && st.status == SP_TRAJ_OK; step++) {
        while (oi < nout && sc->output_steps[oi] <= step) {
            if (out) memcpy(out + (size_t)oi * NS, st.x, sizeof(int32_t) * NS);
            oi++;
        }
        nsm_window(t, &st, step, selection);
    }
    while (out && oi < nout) {
        memcpy(out + (size_t)oi * NS, st.x, sizeof(int32_t) * NS);
        oi++;
    }
    ev[0] = st.nrx;
    ev[1] = st.ndf;
    const int status = st.status;
    nsm_state_free(&st);
    return status;
}

int spo_nsm_trajectory(const sp_scenario *sc, const uint32_t *u0, uint64_t seed, int32_t selection,
                       int32_t *out, int64_t *ev) {
    nsm_tables_t t;
    tables_build(sc, &t);
    int st = nsm_run(&t, u0, seed, selection, out, ev);
    tables_free(&t);
    return st;
}

typedef struct {
    const nsm_tables_t *t;
    const uint32_t *u0;
    const uint64_t *seeds;
    int ntraj, selection;
    int32_t *out;
    int64_t *ev;
    int32_t *status;
    int next;
    pthread_mutex_t mu;
} ens_t;

static void *ens_worker(void *arg) {
    ens_t *e = (ens_t *)arg;
    const size_t per = (size_t)e->t->sc->num_outputs * e->t->N * e->t->S;
    for (;;) {
        pthread_mutex_lock(&e->mu);
        int j = e->next++;
        pthread_mutex_unlock(&e->mu);
        if (j >= e->ntraj) break;
        int st = nsm_run(e->t, e->u0, e->seeds[j], e->selection, e->out ? e->out + per * j : NULL,
                         e->ev + 2 * j);
        if (e->status) e->status[j] = st;
    }
    return NULL;
}

int spo_nsm_ensemble(const sp_scenario *sc, const uint32_t *u0, const uint64_t *seeds,
                     int32_t ntraj, int32_t selection, int32_t threads, int32_t *out,
                     int64_t *ev, int32_t *status) {
    nsm_tables_t t;
    tables_build(sc, &t);
    if (threads <= 0) threads = (int)sysconf(_SC_NPROCESSORS_ONLN);
    if (threads > ntraj) threads = ntraj;
    if (threads < 1) threads = 1;
    ens_t e = {&t, u0, seeds, ntraj, selection, out, ev, status, 0, PTHREAD_MUTEX_INITIALIZER};
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    for (int i = 0; i < threads; i++) pthread_create(&th[i], NULL, ens_worker, &e);
    for (int i = 0; i < threads; i++) pthread_join(th[i], NULL);
    free(th);
    tables_free(&t);
    return threads;
}

/* ------------------------------------------------------------------------
 * Moving domain with species: the SDPD flow (shared by all trajectories)
 * and, every step, fresh diffusion tables, volumes and event queues.
 * ------------------------------------------------------------------------ */
typedef struct {
    const nsm_tables_t *t;
    nsm_state_t *st;
    int ntraj, step, selection, next;
    pthread_mutex_t mu;
} cstep_t;

static void *coupled_worker(void *arg) {
    cstep_t *c = (cstep_t *)arg;
    for (;;) {
        pthread_mutex_lock(&c->mu);
        const int j = c->next++;
        pthread_mutex_unlock(&c->mu);
        if (j >= c->ntraj) break;
        if (c->st[j].status != SP_TRAJ_OK) continue;
        nsm_build(c->t, &c->st[j], c->t->sc->dt * (double)c->step, (uint32_t)c->step);
        nsm_window(c->t, &c->st[j], c->step, c->selection);
    }
    return NULL;
}

int spo_coupled_ensemble(const sp_scenario *sc, const uint32_t *u0, const uint64_t *seeds,
                         int32_t ntraj, int32_t selection, int32_t precision, int32_t mode,
                         int32_t kmax, int32_t threads, int32_t *out, int64_t *ev,
                         int32_t *status, double *px, double *prho, double *chem_out) {
    const int N = sc->num_particles, S = sc->num_species, R = sc->num_reactions;
    int nth = threads <= 0 ? (int)sysconf(_SC_NPROCESSORS_ONLN) : threads;
    if (nth > ntraj) nth = ntraj;
    if (nth < 1) nth = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nth);
    const size_t NS = (size_t)N * S;
    double *x = (double *)malloc(sizeof(double) * 3 * N), *v = (double *)calloc(3 * N, sizeof(double));
    double *vt = (double *)calloc(3 * N, sizeof(double)), *F = (double *)calloc(3 * N, sizeof(double));
    double *Fbp = (double *)calloc(3 * N, sizeof(double)), *rho = (double *)malloc(sizeof(double) * N);
    double *Frho = (double *)calloc(N, sizeof(double));
    memcpy(x, sc->x, sizeof(double) * 3 * N);
    if (sc->v) memcpy(v, sc->v, sizeof(double) * 3 * N);
    memcpy(rho, sc->rho, sizeof(double) * N);
    spo_f32_state fs = {(float *)malloc(sizeof(float) * 3 * N), (float *)malloc(sizeof(float) * 3 * N),
                        (float *)malloc(sizeof(float) * N), 0};
    spo_sdpd_lists L;
    L.count = (int32_t *)calloc(N, sizeof(int32_t));
    L.idx = (int32_t *)malloc(sizeof(int32_t) * (size_t)N * kmax);
    L.dij = (double *)malloc(sizeof(double) * (size_t)N * kmax);
    nsm_tables_t t;
    memset(&t, 0, sizeof(t));
    t.sc = sc;
    t.N = N;
    t.S = S;
    t.R = R;
    t.T = sc->num_types;
    t.K = kmax;
    t.cnt = L.count;
    t.idx = L.idx;
    t.cdf = (float *)calloc(NS * kmax, sizeof(float));
    t.ddiag = (float *)calloc(NS, sizeof(float));
    t.vol = (float *)malloc(sizeof(float) * N);
    t.ivol = (float *)malloc(sizeof(float) * N);
    t.rate = (float *)malloc(sizeof(float) * (R > 0 ? R : 1));
    for (int r = 0; r < R; r++) t.rate[r] = (float)sc->rxn_rate[r];
    nsm_state_t *st = (nsm_state_t *)malloc(sizeof(nsm_state_t) * ntraj);
    for (int j = 0; j < ntraj; j++) nsm_state_init(&st[j], &t, u0, seeds[j]);
    spo_chem ch;
    ch.C = sc->enable_pde ? (double *)calloc(NS, sizeof(double)) : NULL;
    ch.Q = sc->enable_pde ? (double *)calloc(NS, sizeof(double)) : NULL;
    ch.nu = (double *)malloc(sizeof(double) * N);
    memcpy(ch.nu, sc->nu, sizeof(double) * N);
    if (ch.C)
        for (size_t e = 0; e < NS; e++) ch.C[e] = (double)u0[e];
    int rc = 0, oi = 0;
    const int nout = sc->num_outputs;
    for (int step = 0; step < sc->num_steps && !rc; step++) {
        while (oi < nout && sc->output_steps[oi] <= step) {
            for (int j = 0; j < ntraj && out; j++)
                memcpy(out + ((size_t)j * nout + oi) * NS, st[j].x, sizeof(int32_t) * NS);
            if (px) memcpy(px + (size_t)oi * 3 * N, x, sizeof(double) * 3 * N);
            if (prho) memcpy(prho + (size_t)oi * N, rho, sizeof(double) * N);
            if (chem_out && ch.C) memcpy(chem_out + (size_t)oi * NS, ch.C, sizeof(double) * NS);
            oi++;
        }
        rc = precision == 64
                 ? spo_sdpd_f64(sc, step, 1, mode, kmax, x, v, vt, rho, F, Fbp, Frho, NULL, &L, &ch,
                                NULL)
                 : spo_sdpd_f32(sc, step, 1, mode, kmax, x, v, vt, rho, F, Fbp, Frho, NULL, &L, &ch,
                                &fs);
        if (rc) break;
        /* nsm_core__initialize_rxn/diff_propensities (simulate_rdme.cpp:113-152)
           with this step's lists and the end-of-step densities */
        spo_diffusion_tables(sc, kmax, L.count, L.idx, L.dij, t.ddiag, t.cdf);
        for (int i = 0; i < N; i++) {
            t.vol[i] = (float)(sc->mass[i] / rho[i]);
            t.ivol[i] = (float)(rho[i] / sc->mass[i]);
        }
        /* nsm_core__initialize_heap at step*dt, then take_step (:53-68);
           trajectories are independent within a step */
        cstep_t cs = {&t, st, ntraj, step, selection, 0, PTHREAD_MUTEX_INITIALIZER};
        if (nth <= 1) {
            coupled_worker(&cs);
        } else {
            for (int i = 0; i < nth; i++) pthread_create(&th[i], NULL, coupled_worker, &cs);
            for (int i = 0; i < nth; i++) pthread_join(th[i], NULL);
        }
    }
    while (!rc && oi < nout) {
        for (int j = 0; j < ntraj && out; j++)
            memcpy(out + ((size_t)j * nout + oi) * NS, st[j].x, sizeof(int32_t) * NS);
        if (px) memcpy(px + (size_t)oi * 3 * N, x, sizeof(double) * 3 * N);
        if (prho) memcpy(prho + (size_t)oi * N, rho, sizeof(double) * N);
        if (chem_out && ch.C) memcpy(chem_out + (size_t)oi * NS, ch.C, sizeof(double) * NS);
        oi++;
    }
    free(ch.C); free(ch.Q); free(ch.nu);
    free(fs.xh); free(fs.xl); free(fs.drho);
    for (int j = 0; j < ntraj; j++) {
        ev[2 * j] = st[j].nrx;
        ev[2 * j + 1] = st[j].ndf;
        if (status) status[j] = st[j].status;
        nsm_state_free(&st[j]);
    }
    free(st);
    free(th);
    free(t.cdf); free(t.ddiag); free(t.vol); free(t.ivol); free(t.rate);
    free(L.count); free(L.idx); free(L.dij);
    free(x); free(v); free(vt); free(F); free(Fbp); free(rho); free(Frho);
    return rc;
}

/* ------------------------------------------------------------------------
 * Deterministic chemistry and boundary conditions
 * ------------------------------------------------------------------------ */
static int bc_hit(const sp_scenario *sc, int b, int i, const double p[3]) {
    const double *bx = sc->bc_box + 6 * b;
    return p[0] >= bx[0] && p[0] <= bx[1] && p[1] >= bx[2] && p[1] <= bx[3] && p[2] >= bx[4] &&
           p[2] <= bx[5] && (sc->bc_type[b] == 0 || sc->bc_type[b] == sc->type[i]);
}

void spo_flow_bcs(const sp_scenario *sc, int i, const double p[3], double v[3], double *nu,
                  double *rho) {
    for (int b = 0; b < sc->num_bcs; b++) {
        const int tg = sc->bc_target[b];
        if (tg >= SP_BC_C || !bc_hit(sc, b, i, p)) continue;
        const double *val = sc->bc_value + 3 * b;
        if (tg == SP_BC_V) { v[0] = val[0]; v[1] = val[1]; v[2] = val[2]; }
        else if (tg == SP_BC_NU) *nu = val[0];
        else *rho = val[0];
    }
}

void spo_chem_half(const sp_scenario *sc, double *C, double *Q, const double *pos, int pstride,
                   int first, int clear_q) {
    const int N = sc->num_particles, S = sc->num_species;
    const double coef = first ? 0.0 : 0.5 * sc->dt;
    for (int i = 0; i < N; i++) {
        double *c = C + (size_t)i * S, *q = Q + (size_t)i * S;
        if (coef != 0.0)
            for (int s = 0; s < S; s++) c[s] = c[s] + q[s] * coef;
        if (sc->num_bcs) {
            const double *p = pos + (size_t)i * pstride;
            for (int b = 0; b < sc->num_bcs; b++) {
                const int tg = sc->bc_target[b];
                if (tg >= SP_BC_C && bc_hit(sc, b, i, p)) c[tg - SP_BC_C] = sc->bc_value[3 * b];
            }
        }
        if (clear_q)
            for (int s = 0; s < S; s++) q[s] = 0.0;
    }
}

void spo_chem_flux(const sp_scenario *sc, const double *C, double *Q, const int32_t *cnt,
                   const int32_t *idx, const double *dist, const double *dwdr, int kstride,
                   const double *mass, const double *rho, double t) {
    const int N = sc->num_particles, S = sc->num_species, R = sc->num_reactions,
              T = sc->num_types;
    const double h = sc->h;
    int *dense = (int *)calloc((size_t)S * (R > 0 ? R : 1), sizeof(int));
    for (int r = 0; r < R; r++)
        for (int64_t q = sc->jcN[r]; q < sc->jcN[r + 1]; q++)
            dense[(size_t)sc->irN[q] * R + r] += sc->prN[q];
    for (int i = 0; i < N; i++) {
        const double *ci = C + (size_t)i * S;
        double *q = Q + (size_t)i * S;
        const double mi = mass[i], ri = rho[i];
        const int ti = sc->type[i];
        for (int k = 0; k < cnt[i]; k++) {
            const size_t o = (size_t)i * kstride + k;
            const double r = dist[o];
            if (r / h > 1.0 || r == 0.0) continue;
            const int j = idx[o];
            const double mj = mass[j], rj = rho[j];
            const double wfd = (1.0 / (r + 0.001 * h)) * dwdr[o];
            const double base = 2.0 * ((mi * mj) / (mi + mj)) * ((ri + rj) / (ri * rj)) * (r * r) *
                                wfd / ((r * r) + 0.01 * h * h);
            const double *cj = C + (size_t)j * S;
            for (int s = 0; s < S; s++)
                q[s] = q[s] + sc->diffusion[s * T + (ti - 1)] * (ci[s] - cj[s]) * base;
        }
        const double vol = mi / ri;
        for (int r = 0; r < R; r++) {
            if (sc->rxn_allowed && !sc->rxn_allowed[(size_t)r * (T + 1) + ti]) continue;
            const double flux = run_program_x(sc, sc->ode_code + sc->ode_code_off[r], sc->ode_consts,
                                              NULL, ci, vol, t, ti, i);
            for (int s = 0; s < S; s++) q[s] = q[s] + (double)dense[(size_t)s * R + r] * flux;
        }
    }
    free(dense);
}

int spo_chem_static(const sp_scenario *sc, const uint32_t *u0, int32_t kmax, double *out) {
    const int N = sc->num_particles, S = sc->num_species;
    int32_t *cnt = (int32_t *)malloc(sizeof(int32_t) * N);
    int32_t *idx = (int32_t *)malloc(sizeof(int32_t) * (size_t)N * kmax);
    double *dist = (double *)malloc(sizeof(double) * (size_t)N * kmax);
    double *dw = (double *)malloc(sizeof(double) * (size_t)N * kmax);
    int rc = spo_neighbors(N, sc->dimension, sc->x, sc->x, sc->h, sc->mass, sc->rho, kmax, cnt, idx,
                           dist, dw, NULL);
    double *C = (double *)calloc((size_t)N * S, sizeof(double));
    double *Q = (double *)calloc((size_t)N * S, sizeof(double));
    for (size_t e = 0; e < (size_t)N * S; e++) C[e] = (double)u0[e];   /* C = u0 */
    int oi = 0;
    const int nout = sc->num_outputs;
    for (int step = 0; step < sc->num_steps && !rc; step++) {
        while (oi < nout && sc->output_steps[oi] <= step) {
            memcpy(out + (size_t)oi * N * S, C, sizeof(double) * N * S);
            oi++;
        }
        spo_chem_half(sc, C, Q, sc->x, 3, step == 0, 1);
        spo_chem_flux(sc, C, Q, cnt, idx, dist, dw, kmax, sc->mass, sc->rho, sc->dt * (double)step);
        spo_chem_half(sc, C, Q, sc->x, 3, 0, 0);
    }
    while (!rc && oi < nout) {
        memcpy(out + (size_t)oi * N * S, C, sizeof(double) * N * S);
        oi++;
    }
    free(cnt); free(idx); free(dist); free(dw); free(C); free(Q);
    return rc;
}
