/*
 * sdpd_oracle_impl.h — TEST INFRASTRUCTURE.  Body of the SDPD oracle,
 * included by sdpd_oracle.c once per arithmetic type (REAL = double/float,
 * SPO_FN = function name).  Restates the engine step
 * (src/simulate.cpp:56-173, src/model.cpp:39-329, src/particle.cpp:150-294)
 * with one thread, in particle order.  Constants are cast to REAL so the
 * float build computes in float throughout.
 *
 * SPO_COMP = 1 (the float build) changes how the state is STORED, not how it
 * is computed: a position is a pair of floats hi + lo advanced by an
 * error-free two-sum, and a density is kept as its deviation from rho0, so
 * that P = P0 (rho/rho0 - 1) = P0 drho/rho0 has no cancellation.  Pair
 * arithmetic stays in float.  With plain float storage the pressure term's
 * sign switch (model.cpp:111-112) is decided on rounding noise and velocities
 * drift 2.8e-4 from FP64 after 1,000 steps of the 1,368-particle dam break;
 * with this storage they agree to 1.2e-6.  The state persists in a
 * spo_f32_state between calls, because hi + lo and rho0 + drho do not
 * round-trip exactly through the double arrays of the interface.  Box tests
 * of boundary conditions and the chemistry read the hi parts; every reader
 * of a density other than the pressure reads the float rho0 + drho.
 */
#define K_(c) ((REAL)(c))

static int SPO_NB(int n, int dim, const REAL *xq, const REAL *xt, const REAL *xql,
                  const REAL *xtl, REAL h, const REAL *mass,
                  const REAL *rho, int kmax, int32_t *count, int32_t *idx, REAL *dist,
                  REAL *dwdr, const REAL *self_d2, REAL *dij) {
    /* same predicate and order as spo_neighbors, in REAL arithmetic */
    REAL lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int d = 0; d < dim; d++) {
        lo[d] = hi[d] = xt[d];
        for (int i = 0; i < n; i++) {
            REAL a = xt[3 * i + d], b = xq[3 * i + d];
            if (a < lo[d]) lo[d] = a;
            if (b < lo[d]) lo[d] = b;
            if (a > hi[d]) hi[d] = a;
            if (b > hi[d]) hi[d] = b;
        }
    }
    const double cs = (double)h * 1.000001;
    int nc[3] = {1, 1, 1};
    for (int d = 0; d < dim; d++) nc[d] = (int)floor(((double)hi[d] - lo[d]) / cs) + 1;
    const long ncell = (long)nc[0] * nc[1] * nc[2];
    int32_t *start = (int32_t *)calloc((size_t)ncell + 1, sizeof(int32_t));
    int32_t *cell = (int32_t *)malloc(sizeof(int32_t) * n);
    int32_t *order = (int32_t *)malloc(sizeof(int32_t) * n);
#define CELLD(p, d) ((d) < dim ? (int)fmin(nc[d] - 1, floor(((double)(p) - lo[d]) / cs)) : 0)
    for (int i = 0; i < n; i++) {
        cell[i] = (int32_t)(((long)CELLD(xt[3 * i], 0) * nc[1] + CELLD(xt[3 * i + 1], 1)) * nc[2] +
                            CELLD(xt[3 * i + 2], 2));
        start[cell[i] + 1]++;
    }
    for (long c = 0; c < ncell; c++) start[c + 1] += start[c];
    int32_t *fill = (int32_t *)malloc(sizeof(int32_t) * ncell);
    memcpy(fill, start, sizeof(int32_t) * ncell);
    for (int i = 0; i < n; i++) order[fill[cell[i]]++] = i;
    free(fill);
    const REAL sq = h * h;
    const REAL alpha = dim == 3 ? K_(105) / (K_(16) * K_(M_PI) * h * h * h)
                     : dim == 2 ? K_(5) / (K_(M_PI) * h * h) : h;
    int rc = 0;
    REAL *cd2 = (REAL *)malloc(sizeof(REAL) * (kmax + 1));
    int32_t *cj = (int32_t *)malloc(sizeof(int32_t) * (kmax + 1));
    for (int i = 0; i < n && !rc; i++) {
        const REAL *q = xq + 3 * i;
        int qc[3];
        for (int d = 0; d < 3; d++) qc[d] = CELLD(q[d], d);
        int m = 0;
        for (int a = qc[0] - 1; a <= qc[0] + 1 && !rc; a++) {
            if (a < 0 || a >= nc[0]) continue;
            for (int b = qc[1] - 1; b <= qc[1] + 1 && !rc; b++) {
                if (b < 0 || b >= nc[1]) continue;
                for (int c = qc[2] - 1; c <= qc[2] + 1 && !rc; c++) {
                    if (c < 0 || c >= nc[2]) continue;
                    long cid = ((long)a * nc[1] + b) * nc[2] + c;
                    for (int32_t t = start[cid]; t < start[cid + 1]; t++) {
                        int j = order[t];
                        const REAL *p = xt + 3 * j;
                        REAL d2 = 0;
                        int d;
                        for (d = 0; d < dim; d++) {
                            REAL tt = q[d] - p[d];
#if SPO_COMP
                            tt = tt + (xql[3 * i + d] - xtl[3 * j + d]);
#endif
                            d2 = d2 + tt * tt;
                            if (d2 > sq) break;
                        }
                        if (self_d2 && j == i) { d2 = self_d2[i]; d = dim; }
                        if (d2 > sq) continue;
                        if (d < dim || d2 == 0) continue;
                        if (SQRT(d2) > h) continue;
                        if (m >= kmax) { rc = -1; break; }
                        int k = m++;
                        while (k > 0 && (d2 < cd2[k - 1] || (d2 == cd2[k - 1] && j < cj[k - 1]))) {
                            cd2[k] = cd2[k - 1];
                            cj[k] = cj[k - 1];
                            k--;
                        }
                        cd2[k] = d2;
                        cj[k] = j;
                    }
                }
            }
        }
        count[i] = m;
        for (int k = 0; k < m; k++) {
            const REAL r = SQRT(cd2[k]);
            const REAL R = r / h;
            idx[(size_t)i * kmax + k] = cj[k];
            dist[(size_t)i * kmax + k] = r;
            dwdr[(size_t)i * kmax + k] = alpha * (K_(-12) * r / (h * h)) * ((K_(1) - R) * (K_(1) - R));
            if (dij) {
                /* D_ij of add_to_neighbor_list (particle.cpp:181-187) with the
                   densities current at the search, operator order kept */
                const int j = cj[k];
                const REAL r2 = cd2[k];
                const REAL ih = K_(1.0) / h;
                const REAL ihsq = ih * ih;
                const REAL dhr = h - r;
                const REAL wfd = K_(-25.066903536973515383) * dhr * dhr * ihsq * ihsq * ihsq * ih;
                dij[(size_t)i * kmax + k] = K_(-2.0) * (mass[i] * mass[j]) / (mass[i] + mass[j]) *
                                            (rho[i] + rho[j]) / (rho[i] * rho[j]) * r2 * wfd /
                                            (r2 + K_(0.01) * h * h);
            }
        }
    }
#undef CELLD
    free(cd2); free(cj); free(start); free(cell); free(order);
    return rc;
}

int SPO_FN(const sp_scenario *sc, int32_t step0, int32_t nsteps, int32_t mode, int32_t kmax,
           double *x_io, double *v_io, double *vt_io, double *rho_io, double *F_io,
           double *Fbp_io, double *Frho_io, int32_t *nbr_count, spo_sdpd_lists *lists,
           spo_chem *chem, spo_f32_state *fs) {
    const int n = sc->num_particles, dim = sc->dimension;
    const REAL h = (REAL)sc->h, dt = (REAL)sc->dt, rho0 = (REAL)sc->rho0, P0 = (REAL)sc->P0;
    const REAL g[3] = {(REAL)sc->gravity[0], (REAL)sc->gravity[1], (REAL)sc->gravity[2]};
    const REAL alpha = dim == 3 ? K_(105) / (K_(16) * K_(M_PI) * h * h * h)
                     : dim == 2 ? K_(5) / (K_(M_PI) * h * h) : h;
    REAL *x = (REAL *)malloc(sizeof(REAL) * 3 * n), *xt = (REAL *)malloc(sizeof(REAL) * 3 * n);
    REAL *v = (REAL *)malloc(sizeof(REAL) * 3 * n), *vt = (REAL *)malloc(sizeof(REAL) * 3 * n);
    REAL *F = (REAL *)malloc(sizeof(REAL) * 3 * n), *Fbp = (REAL *)malloc(sizeof(REAL) * 3 * n);
    REAL *rho = (REAL *)malloc(sizeof(REAL) * n), *orho = (REAL *)malloc(sizeof(REAL) * n);
    REAL *Frho = (REAL *)malloc(sizeof(REAL) * n), *m = (REAL *)malloc(sizeof(REAL) * n);
    REAL *nu = (REAL *)malloc(sizeof(REAL) * n), *nrm = (REAL *)malloc(sizeof(REAL) * 3 * n);
    REAL *sd2 = (REAL *)malloc(sizeof(REAL) * n);
    REAL *ndist = (REAL *)malloc(sizeof(REAL) * (size_t)n * kmax);
    REAL *ndw = (REAL *)malloc(sizeof(REAL) * (size_t)n * kmax);
    int32_t *nidx = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * kmax);
    int32_t *ncnt = (int32_t *)malloc(sizeof(int32_t) * n);
    REAL *ndij = lists ? (REAL *)malloc(sizeof(REAL) * (size_t)n * kmax) : NULL;
    /* double copies for the chemistry and the boundary conditions */
    double *pd = (double *)malloc(sizeof(double) * 3 * n);
    double *dd = chem ? (double *)malloc(sizeof(double) * (size_t)n * kmax) : NULL;
    double *wd = chem ? (double *)malloc(sizeof(double) * (size_t)n * kmax) : NULL;
    double *md = chem ? (double *)malloc(sizeof(double) * n) : NULL;
    double *rd = chem ? (double *)malloc(sizeof(double) * n) : NULL;
    const int do_chem = chem && chem->C && sc->enable_pde && sc->num_species > 0;
#if SPO_COMP
    /* x, xt hold the hi parts, xl, xtl the lo parts; rho, orho hold
       deviations from rho0 and rf, orf the float densities rho0 + deviation */
    REAL *xl = (REAL *)malloc(sizeof(REAL) * 3 * n), *xtl = (REAL *)malloc(sizeof(REAL) * 3 * n);
    REAL *rf = (REAL *)malloc(sizeof(REAL) * n), *orf = (REAL *)malloc(sizeof(REAL) * n);
#else
    REAL *xl = NULL, *xtl = NULL, *rf = rho, *orf = orho;
#endif
    for (int i = 0; i < 3 * n; i++) {
        x[i] = (REAL)x_io[i]; v[i] = (REAL)v_io[i]; vt[i] = (REAL)vt_io[i];
        F[i] = (REAL)F_io[i]; Fbp[i] = (REAL)Fbp_io[i];
#if SPO_COMP
        xl[i] = (REAL)(x_io[i] - (double)x[i]);
#endif
    }
    for (int i = 0; i < n; i++) {
#if SPO_COMP
        rho[i] = (REAL)(rho_io[i] - sc->rho0);
#else
        rho[i] = (REAL)rho_io[i];
#endif
        Frho[i] = (REAL)Frho_io[i];
        m[i] = (REAL)sc->mass[i]; nu[i] = (REAL)(chem && chem->nu ? chem->nu[i] : sc->nu[i]);
    }
#if SPO_COMP
    if (fs && fs->valid) {
        memcpy(x, fs->xh, sizeof(REAL) * 3 * n);
        memcpy(xl, fs->xl, sizeof(REAL) * 3 * n);
        memcpy(rho, fs->drho, sizeof(REAL) * n);
    }
    for (int i = 0; i < n; i++) rf[i] = rho0 + rho[i];
#else
    (void)fs;
#endif
    int rc = 0;
    for (int step = step0; step < step0 + nsteps && !rc; step++) {
        memcpy(xt, x, sizeof(REAL) * 3 * n);            /* kd-tree points of this step */
#if SPO_COMP
        memcpy(xtl, xl, sizeof(REAL) * 3 * n);
#endif
        /* substep 0: take_step1 (simulate.cpp:56-109) */
        for (int i = 0; i < n; i++) {
            for (int d = 0; d < 3; d++)
                if (isnan((double)x[3 * i + d]) || !isfinite((double)x[3 * i + d]) ||
                    isnan((double)v[3 * i + d]) || !isfinite((double)v[3 * i + d])) rc = 2;
            if (isnan((double)rho[i]) || !isfinite((double)rho[i])) rc = 2;
            if (!sc->fixed[i] && !sc->static_domain) {
                for (int d = 0; d < 3; d++) {
                    v[3 * i + d] = v[3 * i + d] + K_(0.5) * dt * F[3 * i + d];
                    vt[3 * i + d] = v[3 * i + d] + K_(0.5) * dt * Fbp[3 * i + d];
#if SPO_COMP
                    {   /* two-sum of hi and the step, renormalised into hi + lo */
                        const REAL a = x[3 * i + d], b = dt * vt[3 * i + d];
                        const REAL s = a + b, bb = s - a;
                        const REAL e = (a - (s - bb)) + (b - bb);
                        const REAL lo = xl[3 * i + d] + e, s2 = s + lo;
                        xl[3 * i + d] = lo - (s2 - s);
                        x[3 * i + d] = s2;
                    }
#else
                    x[3 * i + d] = x[3 * i + d] + dt * vt[3 * i + d];
#endif
                }
                rho[i] = rho[i] + K_(0.5) * dt * Frho[i];
            }
            if (sc->num_bcs) {   /* applyBoundaryConditions after the predictor */
                double p[3] = {(double)x[3 * i], (double)x[3 * i + 1], (double)x[3 * i + 2]};
                double vv[3] = {(double)v[3 * i], (double)v[3 * i + 1], (double)v[3 * i + 2]};
#if SPO_COMP
                const double rin = sc->rho0 + (double)rho[i];
#else
                const double rin = (double)rho[i];
#endif
                double nn = (double)nu[i], rr = rin;
                spo_flow_bcs(sc, i, p, vv, &nn, &rr);
                for (int d = 0; d < 3; d++) v[3 * i + d] = (REAL)vv[d];
                nu[i] = (REAL)nn;
#if SPO_COMP
                if (rr != rin) rho[i] = (REAL)(rr - sc->rho0);
#else
                rho[i] = (REAL)rr;
#endif
            }
            for (int d = 0; d < 3; d++) { F[3 * i + d] = g[d]; Fbp[3 * i + d] = 0; }
            Frho[i] = 0;
            orho[i] = rho[i];
        }
        if (rc) break;
#if SPO_COMP
        for (int i = 0; i < n; i++) orf[i] = rf[i] = rho0 + rho[i];
#endif
        if (do_chem) {
            for (int e = 0; e < 3 * n; e++) pd[e] = (double)x[e];
            spo_chem_half(sc, chem->C, chem->Q, pd, 3, step == 0, 1);
        }
        /* neighbour lists used by substeps 1-2 (particle.cpp:240-294): at step 0
           from the unmoved points; later from moved queries against the
           start-of-step points (mode 2) or against moved points */
        const REAL *q = (step == 0) ? xt : x;
        const REAL *tp = (step == 0 || (mode & 2)) ? xt : x;
        const REAL *ql = (step == 0) ? xtl : xl;
        const REAL *tpl = (step == 0 || (mode & 2)) ? xtl : xl;
        /* mode 4: a moved particle meets its own start-of-step point at the
           predictor displacement |dt vt| (resolved even where positions
           round to the same value).  The reference's double positions drop
           the pair when the step rounds away (below half a unit in the last
           place of every coordinate); such steps are rounding noise, e.g. the
           background-pressure force of a symmetric lattice neighbourhood, and
           a float step's noise lies far above double resolution, so no float
           rule can reproduce that choice.  It matters: the FP64 flow with
           this mode and with mode 2 differ by 1.2e-4 in velocity after 1,000
           steps of the 1,368-particle dam break. */
        const int selfmode = (mode & 4) && (mode & 2) && step != 0;
        if (selfmode)
            for (int i = 0; i < n; i++) {
                REAL s2 = 0;
                if (!sc->fixed[i] && !sc->static_domain) {
                    const REAL a = dt * vt[3 * i], b = dt * vt[3 * i + 1], c = dt * vt[3 * i + 2];
                    s2 = a * a;
                    if (dim > 1) s2 = s2 + b * b;
                    if (dim > 2) s2 = s2 + c * c;
                }
                sd2[i] = s2;
            }
        if (SPO_NB(n, dim, q, tp, ql, tpl, h, m, rf, kmax, ncnt, nidx, ndist, ndw, selfmode ? sd2 : NULL,
                   ndij)) {
            rc = -1;
            break;
        }
        /* substep 1: pairwiseForce (model.cpp:39-191) */
        for (int i = 0; i < n; i++) {
            #if SPO_COMP
            const REAL Pi = P0 * (rho[i] / rho0);
#else
            const REAL Pi = P0 * (rho[i] / rho0 - K_(1.0));
#endif
            REAL Fi[3] = {F[3 * i], F[3 * i + 1], F[3 * i + 2]};
            REAL Fb[3] = {Fbp[3 * i], Fbp[3 * i + 1], Fbp[3 * i + 2]};
            REAL Fr = Frho[i];
            for (int k = 0; k < ncnt[i]; k++) {
                const int j = nidx[(size_t)i * kmax + k];
                const REAL r = ndist[(size_t)i * kmax + k];
                const REAL R = r / h;
                if (R > K_(1.0) || r == 0) continue;
                const REAL dWdr = ndw[(size_t)i * kmax + k];
                REAL dx[3] = {0, 0, 0}, dv[3] = {0, 0, 0}, dvdx = 0;
                for (int d = 0; d < dim; d++) {
                    dx[d] = x[3 * i + d] - x[3 * j + d];
#if SPO_COMP
                    dx[d] = dx[d] + (xl[3 * i + d] - xl[3 * j + d]);
#endif
                    dv[d] = v[3 * i + d] - v[3 * j + d];
                    dvdx = dvdx + dv[d] * dx[d];
                }
#if SPO_COMP
                const REAL Pj = P0 * (rho[j] / rho0);
#else
                const REAL Pj = P0 * (rho[j] / rho0 - K_(1.0));
#endif
                REAL pg = Pi / (rf[i] * rf[i]) + Pj / (rf[j] * rf[j]);
                if (pg < 0) pg = -Pi / (rf[i] * rf[i]) + Pj / (rf[j] * rf[j]);
                const REAL rh = r + K_(0.001) * h;
                const REAL fp = K_(-1.0) * m[j] * pg * dWdr / rh;
                const REAL fv = m[j] * (K_(2.0) * (nu[i] * nu[j]) / (nu[i] + nu[j])) * (K_(1) / rh) * dWdr /
                                (rf[i] * rf[j]);
                const REAL vi = m[i] / rf[i], vj = m[j] / rf[j];
                const REAL ss = vi * vi + vj * vj;
                const REAL fbp = K_(-10.0) * P0 * (K_(1.0) / m[i]) * ss * dWdr / rh;
                REAL ft[3];
                for (int a = 0; a < 3; a++) {
                    REAL tt0 = K_(0.5) * ((rf[i] * v[3 * i + a] * (vt[3 * i + 0] - v[3 * i + 0])) +
                                         (rf[j] * v[3 * j + a] * (vt[3 * j + 0] - v[3 * j + 0])));
                    REAL tt1 = K_(0.5) * ((rf[i] * v[3 * i + a] * (vt[3 * i + 1] - v[3 * i + 1])) +
                                         (rf[j] * v[3 * j + a] * (vt[3 * j + 1] - v[3 * j + 1])));
                    REAL tt2 = K_(0.5) * ((rf[i] * v[3 * i + a] * (vt[3 * i + 2] - v[3 * i + 2])) +
                                         (rf[j] * v[3 * j + a] * (vt[3 * j + 2] - v[3 * j + 2])));
                    ft[a] = (K_(1.0) / m[i]) * ss * (tt0 * dx[0] + tt1 * dx[1] + tt2 * dx[2]) * dWdr / rh;
                }
                for (int d = 0; d < dim; d++) {
                    Fi[d] = Fi[d] + (fp * dx[d] + fv * dv[d] + ft[d]);
                    Fb[d] = Fb[d] + fbp * dx[d];
                }
                const REAL tvi = (v[3 * i] - vt[3 * i]) * dx[0] + (v[3 * i + 1] - vt[3 * i + 1]) * dx[1] +
                                 (v[3 * i + 2] - vt[3 * i + 2]) * dx[2];
                const REAL tvj = (v[3 * j] - vt[3 * j]) * dx[0] + (v[3 * j + 1] - vt[3 * j + 1]) * dx[1] +
                                 (v[3 * j + 2] - vt[3 * j + 2]) * dx[2];
                /* the reference's middle term (model.cpp:144) is multiplied by
                   0.0 and omitted here */
                Fr = Fr + rf[i] * vj * dvdx * (K_(1) / rh) * dWdr -
                     vj * (rf[i] * tvi + rf[j] * tvj) * (K_(1.0) / rh) * dWdr;
            }
            for (int d = 0; d < 3; d++) { F[3 * i + d] = Fi[d]; Fbp[3 * i + d] = Fb[d]; }
            Frho[i] = Fr;
        }
        if (do_chem) {   /* the chemistry part of pairwiseForce (model.cpp:151-189) */
            for (size_t e = 0; e < (size_t)n * kmax; e++) {
                dd[e] = (double)ndist[e];
                wd[e] = (double)ndw[e];
            }
            for (int i = 0; i < n; i++) { md[i] = (double)m[i]; rd[i] = (double)rf[i]; }
            spo_chem_flux(sc, chem->C, chem->Q, ncnt, nidx, dd, wd, kmax, md, rd,
                          sc->dt * (double)step);
        }
        /* substep 2: take_step2 (simulate.cpp:132-173) */
        const REAL *rb = (mode & 1) ? rf : orf;     /* density read by the BVF pass */
        for (int i = 0; i < n; i++) {
            const int fluid = !sc->fixed[i] && !sc->static_domain;
            const int wall = sc->fixed[i] && !sc->static_domain;
            if (fluid)
                for (int d = 0; d < 3; d++) v[3 * i + d] = v[3 * i + d] + K_(0.5) * dt * F[3 * i + d];
            if ((fluid || wall) && step % 20 == 0) {            /* filterDensity, model.cpp:194-233 */
                REAL num = 0, den = 0;
                for (int k = 0; k < ncnt[i]; k++) {
                    const int j = nidx[(size_t)i * kmax + k];
                    const REAL r = ndist[(size_t)i * kmax + k];
                    const REAL R = r / h;
                    if (R > K_(1.0) || r == 0) continue;
                    const REAL omr = K_(1) - R;
                    const REAL W = alpha * ((K_(1) + K_(3) * R) * (omr * omr * omr));
                    num = num + orho[j] * W;
                    den = den + W;
                }
                rho[i] = num / den;
            }
            if (fluid) {
                rho[i] = rho[i] + K_(0.5) * dt * Frho[i];
                /* computeBoundaryVolumeFraction, model.cpp:236-313 */
                REAL nw[3] = {0, 0, 0}, vos = 0, vtot = 0;
                for (int d = 0; d < dim; d++) vt[3 * i + d] = 0;
                for (int k = 0; k < ncnt[i]; k++) {
                    const int j = nidx[(size_t)i * kmax + k];
                    const REAL r = ndist[(size_t)i * kmax + k];
                    const REAL R = r / h;
                    if (R > K_(1.0) || r == 0) continue;
                    const REAL omr = K_(1) - R;
                    const REAL W = alpha * ((K_(1) + K_(3) * R) * (omr * omr * omr));
                    const REAL dWdr = ndw[(size_t)i * kmax + k];
                    REAL dx[3] = {0, 0, 0};
                    for (int d = 0; d < dim; d++) {
                        dx[d] = x[3 * i + d] - x[3 * j + d];
#if SPO_COMP
                        dx[d] = dx[d] + (xl[3 * i + d] - xl[3 * j + d]);
#endif
                    }
                    const REAL vj = m[j] / rb[j];
                    const REAL vv = vj * vj;
                    if (sc->fixed[j]) vos = vos + vv * W;
                    vtot = vtot + vv * W;
                    if (sc->fixed[j])
                        for (int a = 0; a < 3; a++) nw[a] = nw[a] + vv * dx[a] * dWdr / (r + K_(0.001) * h);
                }
                for (int a = 0; a < 3; a++) nw[a] = nw[a] / vtot;
                const REAL nn = SQRT(nw[0] * nw[0] + nw[1] * nw[1] + nw[2] * nw[2]);
                for (int a = 0; a < 3; a++) nrm[3 * i + a] = -nw[a] / nn;
                const REAL phi = FABS(vos / vtot);
                /* applyBoundaryVolumeFraction, model.cpp:316-329 */
                const REAL vdn = v[3 * i] * nrm[3 * i] + v[3 * i + 1] * nrm[3 * i + 1] +
                                 v[3 * i + 2] * nrm[3 * i + 2];
                if (phi >= K_(0.5))
                    for (int d = 0; d < dim; d++)
                        v[3 * i + d] = -v[3 * i + d] + K_(2.0) * FMAX(K_(0.0), vdn) * nrm[3 * i + d];
            }
            if (sc->num_bcs) {   /* applyBoundaryConditions after the corrector */
                double p[3] = {(double)x[3 * i], (double)x[3 * i + 1], (double)x[3 * i + 2]};
                double vv[3] = {(double)v[3 * i], (double)v[3 * i + 1], (double)v[3 * i + 2]};
#if SPO_COMP
                const double rin = sc->rho0 + (double)rho[i];
#else
                const double rin = (double)rho[i];
#endif
                double nn = (double)nu[i], rr = rin;
                spo_flow_bcs(sc, i, p, vv, &nn, &rr);
                for (int d = 0; d < 3; d++) v[3 * i + d] = (REAL)vv[d];
                nu[i] = (REAL)nn;
#if SPO_COMP
                if (rr != rin) rho[i] = (REAL)(rr - sc->rho0);
#else
                rho[i] = (REAL)rr;
#endif
            }
#if SPO_COMP
            rf[i] = rho0 + rho[i];
#endif
        }
        if (do_chem) {
            for (int e = 0; e < 3 * n; e++) pd[e] = (double)x[e];
            spo_chem_half(sc, chem->C, chem->Q, pd, 3, 0, 0);
        }
    }
    for (int i = 0; i < 3 * n; i++) {
        x_io[i] = x[i]; v_io[i] = v[i]; vt_io[i] = vt[i]; F_io[i] = F[i]; Fbp_io[i] = Fbp[i];
#if SPO_COMP
        x_io[i] = (double)x[i] + (double)xl[i];
#endif
    }
    for (int i = 0; i < n; i++) { rho_io[i] = rf[i]; Frho_io[i] = Frho[i]; }
#if SPO_COMP
    if (fs) {
        memcpy(fs->xh, x, sizeof(REAL) * 3 * n);
        memcpy(fs->xl, xl, sizeof(REAL) * 3 * n);
        memcpy(fs->drho, rho, sizeof(REAL) * n);
        fs->valid = 1;
    }
    free(xl); free(xtl); free(rf); free(orf);
#endif
    if (nbr_count) memcpy(nbr_count, ncnt, sizeof(int32_t) * n);
    if (lists) {
        /* the lists of the last step, as the NSM of that step reads them */
        memcpy(lists->count, ncnt, sizeof(int32_t) * n);
        memcpy(lists->idx, nidx, sizeof(int32_t) * (size_t)n * kmax);
        for (size_t e = 0; e < (size_t)n * kmax; e++) lists->dij[e] = (double)ndij[e];
    }
    if (chem && chem->nu)
        for (int i = 0; i < n; i++) chem->nu[i] = (double)nu[i];
    free(ndij); free(pd); free(dd); free(wd); free(md); free(rd);
    free(x); free(xt); free(v); free(vt); free(F); free(Fbp); free(rho); free(orho); free(Frho);
    free(m); free(nu); free(nrm); free(ndist); free(ndw); free(nidx); free(ncnt); free(sd2);
    return rc;
}
#undef K_
