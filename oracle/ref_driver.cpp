/*
 * ref_driver.cpp — TEST INFRASTRUCTURE (oracle).  Project-written driver that
 * links the UNMODIFIED SpatialPy C++ engine sources (compiled by
 * oracle/build_ref.sh into oracle/_ref/) and exposes them through a small C
 * API for the parity tests and the CPU baseline.  Nothing in the product
 * links or loads this file.
 *
 * It replaces the code that Solver.compile() would generate from
 * propensity_file_template.cpp (main at :101-142): the particle set-up of
 * init_all_particles (:73-90), the mass-action propensity functions
 * (solver.py:344-373 from reaction.py:260-313), the mass-action ODE rates of
 * the deterministic chemistry (solver.py:160-190, reaction.py:297-303),
 * get_next_output (solver.py:290-299), applyBoundaryConditions as
 * boundarycondition.py:121-167 generates it (one if-block per condition, in
 * order), and `rng`/`debug_flag`.  The step loop replays run_simulation
 * (src/simulate_threads.cpp:232-281) with one worker thread and no output
 * thread: per step buildKDTree, take_step substeps 0,1,2 over all particles
 * in vector order, then simulate_rdme.
 */
#include <algorithm>
#include <chrono>
#include <climits>
#include <unistd.h>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <vector>
#include <random>

#include "particle_system.hpp"
#include "simulate.hpp"
#include "simulate_rdme.hpp"
#include "model.hpp"
#include "output.hpp"
#include "propensities.hpp"
#include "spgpu.h"

int debug_flag = 0;
std::mt19937_64 rng;

namespace Spatialpy {
void buildKDTree(ParticleSystem *system);   /* simulate_threads.cpp:80 */
double *parameters = nullptr;

namespace {
constexpr int kMaxRxn = 64;
int g_R = 0, g_T = 0;
int g_kind[kMaxRxn];
double g_k[kMaxRxn];
int g_a[kMaxRxn], g_b[kMaxRxn];
std::vector<uint8_t> g_allowed;   /* [R*(T+1)] */
std::vector<unsigned int> g_outsteps;
size_t g_outidx = 0;
/* boundary conditions: box [6], type (0 = any), target SP_BC_*, value [3] */
int g_nbc = 0;
std::vector<double> g_bc_box, g_bc_val;
std::vector<int> g_bc_type, g_bc_target;

/* Mass-action propensity with the operator order of the generated C++
 * (e.g. "k_birth*vol", "k*A*B/vol"); x is the engine's unsigned int* xx read
 * as int like the generated functions' `const int *x`. */
template <int R>
double massaction(const unsigned int *xu, double, double vol, double *, int sd) {
    const int *x = reinterpret_cast<const int *>(xu);
    if (!g_allowed.empty() && !g_allowed[(size_t)R * (g_T + 1) + sd]) return 0.0;
    const double k = g_k[R];
    switch (g_kind[R]) {
        case SP_RXN_ZERO:   return k * vol;
        case SP_RXN_FIRST:  return k * x[g_a[R]];
        case SP_RXN_SECOND: return k * x[g_a[R]] * x[g_b[R]] / vol;
        default:            return k * x[g_a[R]] * (x[g_a[R]] - 1) / vol;
    }
}

/* The ODE rate of a mass-action reaction on concentrations, as the
 * generated det<name> function returns it: "k", "k * A", "k * A * B",
 * "k * A * A" (reaction.py:297-303), 0 outside restrict_to types. */
template <int R>
double chem_massaction(double *x, double, double, double *, int sd) {
    if (!g_allowed.empty() && !g_allowed[(size_t)R * (g_T + 1) + sd]) return 0.0;
    const double k = g_k[R];
    switch (g_kind[R]) {
        case SP_RXN_ZERO:   return k;
        case SP_RXN_FIRST:  return k * x[g_a[R]];
        case SP_RXN_SECOND: return k * x[g_a[R]] * x[g_b[R]];
        default:            return k * x[g_a[R]] * x[g_a[R]];
    }
}

template <int... Is> struct Table {
    static PropensityFun *make() {
        static PropensityFun t[] = {(PropensityFun)&massaction<Is>...};
        return t;
    }
    static ChemRxnFun *make_chem() {
        static ChemRxnFun t[] = {(ChemRxnFun)&chem_massaction<Is>...};
        return t;
    }
};
template <int N, int... Is> struct Gen : Gen<N - 1, N - 1, Is...> {};
template <int... Is> struct Gen<0, Is...> { using type = Table<Is...>; };
}  // namespace

unsigned int get_next_output(ParticleSystem *) {
    if (g_outidx < g_outsteps.size()) return g_outsteps[g_outidx++];
    return 0xffffffffu;
}
void applyBoundaryConditions(Particle *me, ParticleSystem *) {
    for (int b = 0; b < g_nbc; b++) {
        const double *bx = &g_bc_box[6 * (size_t)b];
        if (!(me->x[0] >= bx[0] && me->x[0] <= bx[1] && me->x[1] >= bx[2] && me->x[1] <= bx[3] &&
              me->x[2] >= bx[4] && me->x[2] <= bx[5]))
            continue;
        if (g_bc_type[b] != 0 && me->type != g_bc_type[b]) continue;
        const double *val = &g_bc_val[3 * (size_t)b];
        const int tg = g_bc_target[b];
        if (tg == SP_BC_V) {
            for (int i = 0; i < 3; i++) me->v[i] = val[i];
        } else if (tg == SP_BC_NU) {
            me->nu = val[0];
        } else if (tg == SP_BC_RHO) {
            me->rho = val[0];
        } else {
            me->C[tg - SP_BC_C] = val[0];
        }
    }
}
}  // namespace Spatialpy

using namespace Spatialpy;

namespace {

struct Built {
    ParticleSystem *sys = nullptr;
    std::vector<size_t> irN, jcN, irG, jcG;
    std::vector<int> prN;
    std::vector<unsigned int> u0;
    std::vector<int> Ndense;
    ~Built() { delete sys; }
};

int load_network(const sp_scenario *sc) {
    if (sc->num_reactions > kMaxRxn) return SP_E_UNSUPPORTED;
    g_R = sc->num_reactions;
    g_T = sc->num_types;
    for (int r = 0; r < g_R; r++) {
        g_kind[r] = sc->rxn_kind[r];
        g_k[r] = sc->rxn_rate[r];
        g_a[r] = sc->rxn_reactants[2 * r];
        g_b[r] = sc->rxn_reactants[2 * r + 1];
    }
    g_allowed.clear();
    if (sc->rxn_allowed) g_allowed.assign(sc->rxn_allowed, sc->rxn_allowed + (size_t)g_R * (g_T + 1));
    g_outsteps.assign(sc->output_steps, sc->output_steps + sc->num_outputs);
    g_outidx = 0;
    g_nbc = sc->num_bcs;
    g_bc_box.assign(sc->bc_box, sc->bc_box + 6 * (size_t)g_nbc);
    g_bc_val.assign(sc->bc_value, sc->bc_value + 3 * (size_t)g_nbc);
    g_bc_type.assign(sc->bc_type, sc->bc_type + g_nbc);
    g_bc_target.assign(sc->bc_target, sc->bc_target + g_nbc);
    return SP_OK;
}

/* Dependency graph as Model.__create_dependency_graph builds it for
 * mass-action models (model.py:187-250): column s lists reactions having s as
 * reactant; column S+r lists reactions whose reactants are touched by r. */
void dep_graph(const sp_scenario *sc, Built &b) {
    const int S = sc->num_species, R = sc->num_reactions;
    std::vector<std::vector<int>> reac(R), touched(R);
    for (int r = 0; r < R; r++) {
        for (int q = 0; q < 2; q++) {
            int a = sc->rxn_reactants[2 * r + q];
            if (a >= 0) reac[r].push_back(a);
        }
        for (int64_t i = sc->jcN[r]; i < sc->jcN[r + 1]; i++) touched[r].push_back((int)sc->irN[i]);
        for (int a : reac[r]) touched[r].push_back(a);
    }
    std::vector<std::vector<char>> G(R, std::vector<char>(S + R, 0));
    for (int s = 0; s < S; s++)
        for (int j = 0; j < R; j++)
            for (int a : reac[j]) if (a == s) G[j][s] = 1;
    for (int r = 0; r < R; r++)
        for (int s : touched[r])
            for (int j = 0; j < R; j++)
                for (int a : reac[j]) if (a == s) G[j][S + r] = 1;
    b.jcG.assign(1, 0);
    for (int c = 0; c < S + R; c++) {
        for (int r = 0; r < R; r++) if (G[r][c]) b.irG.push_back(r);
        b.jcG.push_back(b.irG.size());
    }
}

/* with_chem: the deterministic chemistry on (Model.enable_pde), its
 * concentrations starting at u0 (propensity_file_template.cpp:77-80). */
int build(const sp_scenario *sc, Built &b, int with_rdme, const uint32_t *chem_u0 = nullptr) {
    int rc = load_network(sc);
    if (rc) return rc;
    const int S = sc->num_species, R = sc->num_reactions, N = sc->num_particles;
    const int with_chem = chem_u0 != nullptr;
    b.sys = new ParticleSystem(sc->num_types, with_chem ? S : 0, with_chem ? R : 0,
                               with_rdme ? S : 0, with_rdme ? R : 0, 0);
    ParticleSystem *sys = b.sys;
    sys->static_domain = sc->static_domain != 0;
    sys->initialized = 0;   /* not set by the constructor (particle.cpp:49-58) */
    sys->dt = sc->dt;
    sys->nt = sc->num_steps;
    sys->h = sc->h;
    sys->rho0 = sc->rho0;
    sys->c0 = sc->c0;
    sys->P0 = sc->P0;
    sys->dimension = sc->dimension;
    for (int d = 0; d < 3; d++) sys->gravity[d] = sc->gravity[d];
    sys->subdomain_diffusion_matrix = sc->diffusion;
    sys->stoch_rxn_propensity_functions = Gen<kMaxRxn>::type::make();
    sys->chem_rxn_rhs_functions = with_chem ? Gen<kMaxRxn>::type::make_chem() : nullptr;
    sys->stoichiometric_matrix = nullptr;
    if (with_chem) {
        /* dense [species][reaction], as solver.py:225-231 writes it */
        b.Ndense.assign((size_t)S * (R > 0 ? R : 1), 0);
        for (int r = 0; r < R; r++)
            for (int64_t q = sc->jcN[r]; q < sc->jcN[r + 1]; q++)
                b.Ndense[(size_t)sc->irN[q] * R + r] += sc->prN[q];
        sys->stoichiometric_matrix = b.Ndense.data();
    }
    sys->species_names = nullptr;
    sys->particles.reserve(N);
    for (int i = 0; i < N; i++) {
        Particle p(sys, (unsigned)i, sc->x[3 * i], sc->x[3 * i + 1], sc->x[3 * i + 2], sc->type[i],
                   sc->nu[i], sc->mass[i], 0.0, sc->rho[i], sc->fixed[i]);
        /* The engine never initialises these before take_step1 reads them
           (particle.cpp:70-83); the oracle starts them at zero. */
        for (int d = 0; d < 3; d++) {
            p.vt[d] = p.F[d] = p.Fbp[d] = p.normal[d] = 0.0;
            p.old_x[d] = p.x[d];
            p.old_v[d] = 0.0;
            if (sc->v) p.v[d] = sc->v[3 * i + d];
        }
        p.Frho = 0.0;
        p.bvf_phi = 0.0;
        p.old_rho = p.rho;
        p.particle_index = (size_t)i;
        if (with_chem)
            for (int s2 = 0; s2 < S; s2++) p.C[s2] = (double)chem_u0[(size_t)i * S + s2];
        sys->particles.emplace_back(p);
    }
    if (with_rdme && S > 0) {
        b.irN.assign(sc->irN, sc->irN + sc->jcN[R]);
        b.jcN.assign(sc->jcN, sc->jcN + R + 1);
        b.prN.assign(sc->prN, sc->prN + sc->jcN[R]);
        dep_graph(sc, b);
    }
    return SP_OK;
}

}  // namespace

extern "C" {

/* Neighbour lists as the engine builds them (kd-tree + find_neighbors). */
int spref_neighbors(const sp_scenario *sc, int32_t kmax, int32_t *count, int32_t *idx,
                    double *dist, double *dwdr, double *dij) {
    Built b;
    int rc = build(sc, b, 0);
    if (rc) return rc;
    ParticleSystem *sys = b.sys;
    buildKDTree(sys);
    Particle *base = &sys->particles[0];
    for (size_t i = 0; i < sys->particles.size(); i++) {
        Particle &p = sys->particles[i];
        p.find_neighbors(sys);
        if ((int)p.neighbors.size() > kmax) return SP_E_INVALID;
        count[i] = (int32_t)p.neighbors.size();
        for (size_t k = 0; k < p.neighbors.size(); k++) {
            const NeighborNode &n = p.neighbors[k];
            idx[i * kmax + k] = (int32_t)(n.data - base);
            dist[i * kmax + k] = n.dist;
            dwdr[i * kmax + k] = n.dWdr;
            dij[i * kmax + k] = n.D_i_j;
        }
    }
    return SP_OK;
}

/*
 * One NSM trajectory on a static domain, seeded like `ssa_sdpd.exe -s seed`
 * (template :127).  out: [num_outputs][N][S] counts at output steps.
 * counters: (total_reactions, total_diffusion).
 */
int spref_nsm(const sp_scenario *sc, const uint32_t *u0, uint64_t seed, int32_t *out,
              int64_t *counters) {
    Built b;
    int rc = build(sc, b, 1);
    if (rc) return rc;
    ParticleSystem *sys = b.sys;
    const int S = sc->num_species, N = sc->num_particles;
    b.u0.assign(u0, u0 + (size_t)N * S);
    rng = std::mt19937_64(seed);
    initialize_rdme(sys, b.irN.data(), b.jcN.data(), b.prN.data(), b.irG.data(), b.jcG.data(),
                    b.u0.data());
    buildKDTree(sys);
    unsigned int next_output = get_next_output(sys);
    int oi = 0;
    for (sys->current_step = 0; sys->current_step < sys->nt; sys->current_step++) {
        if (sys->current_step >= next_output && oi < sc->num_outputs) {
            std::memcpy(out + (size_t)oi * N * S, b.u0.data(), sizeof(uint32_t) * N * S);
            oi++;
            next_output = get_next_output(sys);
        }
        if (!sys->static_domain) return SP_E_UNSUPPORTED;
        if (sys->current_step == 0)
            for (auto &p : sys->particles) p.find_neighbors(sys);
        simulate_rdme(sys, sys->current_step);
    }
    if (oi < sc->num_outputs) {
        std::memcpy(out + (size_t)oi * N * S, b.u0.data(), sizeof(uint32_t) * N * S);
        oi++;
    }
    counters[0] = sys->total_reactions;
    counters[1] = sys->total_diffusion;
    return SP_OK;
}

/*
 * CPU baseline: one static-domain NSM trajectory of the unmodified engine,
 * timing only the event loop (simulate_rdme of simulate_rdme.cpp:53-68,
 * i.e. nsm_core__take_step) over steps [timed_from, nt).  The set-up
 * (particles, kd-tree, neighbour lists, initialize_rdme, the first queue
 * build) and the untimed steps before timed_from are excluded, as the GPU
 * figure excludes them.  counters: (reactions, diffusions) in the timed
 * steps; *seconds: their wall time (steady clock).
 */
int spref_nsm_bench(const sp_scenario *sc, const uint32_t *u0, uint64_t seed, int32_t timed_from,
                    int64_t *counters, double *seconds) {
    Built b;
    int rc = build(sc, b, 1);
    if (rc) return rc;
    ParticleSystem *sys = b.sys;
    if (!sys->static_domain) return SP_E_UNSUPPORTED;
    if (timed_from < 1 || timed_from >= (int)sc->num_steps) return SP_E_INVALID;
    const int S = sc->num_species, N = sc->num_particles;
    b.u0.assign(u0, u0 + (size_t)N * S);
    rng = std::mt19937_64(seed);
    initialize_rdme(sys, b.irN.data(), b.jcN.data(), b.prN.data(), b.irG.data(), b.jcG.data(),
                    b.u0.data());
    buildKDTree(sys);
    for (auto &p : sys->particles) p.find_neighbors(sys);
    long long r0 = 0, d0 = 0;
    auto t0 = std::chrono::steady_clock::now();
    for (sys->current_step = 0; sys->current_step < sys->nt; sys->current_step++) {
        if ((int)sys->current_step == timed_from) {
            r0 = sys->total_reactions;
            d0 = sys->total_diffusion;
            t0 = std::chrono::steady_clock::now();
        }
        simulate_rdme(sys, sys->current_step);
    }
    const auto t1 = std::chrono::steady_clock::now();
    counters[0] = sys->total_reactions - r0;
    counters[1] = sys->total_diffusion - d0;
    *seconds = std::chrono::duration<double>(t1 - t0).count();
    return SP_OK;
}

/*
 * Deterministic chemistry (Model.enable_pde) on any domain: the engine's
 * substeps over [0, nt) with the stochastic part off.  out: [num_outputs][N][S]
 * concentrations C at the output steps.
 */
int spref_chem(const sp_scenario *sc, const uint32_t *u0, double *out) {
    Built b;
    int rc = build(sc, b, 0, u0);
    if (rc) return rc;
    ParticleSystem *sys = b.sys;
    const int S = sc->num_species, N = sc->num_particles;
    unsigned int next_output = get_next_output(sys);
    int oi = 0;
    auto snap = [&]() {
        for (int i = 0; i < N; i++)
            for (int s2 = 0; s2 < S; s2++)
                out[((size_t)oi * N + i) * S + s2] = sys->particles[i].C[s2];
        oi++;
    };
    for (sys->current_step = 0; sys->current_step < sys->nt; sys->current_step++) {
        buildKDTree(sys);
        if (sys->current_step >= next_output && oi < sc->num_outputs) {
            snap();
            next_output = get_next_output(sys);
        }
        for (unsigned sub = 0; sub < 3; sub++)
            for (auto &p : sys->particles) take_step(&p, sys, sys->current_step, sub);
    }
    while (oi < sc->num_outputs) snap();
    return SP_OK;
}

/*
 * A moving domain with stochastic species: per step the kd-tree, the SDPD
 * substeps and simulate_rdme, which on a non-static domain rebuilds the
 * propensities and the queue (simulate_rdme.cpp:53-68).  out:
 * [num_outputs][N][S] counts at the output steps; counters: (reactions,
 * diffusions).
 */
int spref_coupled(const sp_scenario *sc, const uint32_t *u0, uint64_t seed, int32_t *out,
                  int64_t *counters) {
    Built b;
    int rc = build(sc, b, 1);
    if (rc) return rc;
    ParticleSystem *sys = b.sys;
    if (sys->static_domain) return SP_E_UNSUPPORTED;
    const int S = sc->num_species, N = sc->num_particles;
    b.u0.assign(u0, u0 + (size_t)N * S);
    rng = std::mt19937_64(seed);
    initialize_rdme(sys, b.irN.data(), b.jcN.data(), b.prN.data(), b.irG.data(), b.jcG.data(),
                    b.u0.data());
    unsigned int next_output = get_next_output(sys);
    int oi = 0;
    for (sys->current_step = 0; sys->current_step < sys->nt; sys->current_step++) {
        buildKDTree(sys);
        if (sys->current_step >= next_output && oi < sc->num_outputs) {
            std::memcpy(out + (size_t)oi * N * S, b.u0.data(), sizeof(uint32_t) * N * S);
            oi++;
            next_output = get_next_output(sys);
        }
        for (unsigned sub = 0; sub < 3; sub++)
            for (auto &p : sys->particles) take_step(&p, sys, sys->current_step, sub);
        simulate_rdme(sys, sys->current_step);
    }
    while (oi < sc->num_outputs) {
        std::memcpy(out + (size_t)oi * N * S, b.u0.data(), sizeof(uint32_t) * N * S);
        oi++;
    }
    counters[0] = sys->total_reactions;
    counters[1] = sys->total_diffusion;
    return SP_OK;
}

/*
 * The engine loop of run_simulation (kd-tree, output, substeps 0-2,
 * simulate_rdme) with the engine's own VTK writer (output.cpp:59-229)
 * writing outputN.vtk into `dir` at the output steps (N counts the files
 * this process has written).  The full-precision state at each output goes
 * to the arrays (any may be NULL): x, v [T][N][3]; rho, bvf_phi, nu [T][N];
 * counts [T][N][S] (stochastic species) and chem [T][N][S] (with enable_pde).
 */
int spref_vtk_run(const sp_scenario *sc, const uint32_t *u0, uint64_t seed,
                  const char *const *names, const char *dir, double *x, double *v, double *rho,
                  double *bvf, double *nu, int32_t *counts, double *chem) {
    Built b;
    const int S = sc->num_species, N = sc->num_particles;
    const int rdme = S > 0;
    int rc = build(sc, b, rdme, sc->enable_pde && S > 0 ? u0 : nullptr);
    if (rc) return rc;
    ParticleSystem *sys = b.sys;
    sys->species_names = names;
    sys->xlo = sys->ylo = sys->zlo = 1e300;
    sys->xhi = sys->yhi = sys->zhi = -1e300;
    for (const auto &p : sys->particles) {
        sys->xlo = std::min(sys->xlo, p.x[0]); sys->xhi = std::max(sys->xhi, p.x[0]);
        sys->ylo = std::min(sys->ylo, p.x[1]); sys->yhi = std::max(sys->yhi, p.x[1]);
        sys->zlo = std::min(sys->zlo, p.x[2]); sys->zhi = std::max(sys->zhi, p.x[2]);
    }
    if (rdme) {
        b.u0.assign(u0, u0 + (size_t)N * S);
        rng = std::mt19937_64(seed);
        initialize_rdme(sys, b.irN.data(), b.jcN.data(), b.prN.data(), b.irG.data(),
                        b.jcG.data(), b.u0.data());
    }
    char cwd[PATH_MAX];
    if (!getcwd(cwd, sizeof(cwd)) || chdir(dir) != 0) return SP_E_INVALID;
    unsigned int next_output = get_next_output(sys);
    int oi = 0;
    auto snap = [&]() {
        output_vtk__sync_step(sys, sys->current_step);
        output_vtk__async_step(sys);
        for (int i = 0; i < N; i++) {
            const Particle &p = sys->particles[i];
            const size_t o = (size_t)oi * N + i;
            for (int d = 0; d < 3; d++) {
                if (x) x[3 * o + d] = p.x[d];
                if (v) v[3 * o + d] = p.v[d];
            }
            if (rho) rho[o] = p.rho;
            if (bvf) bvf[o] = p.bvf_phi;
            if (nu) nu[o] = p.nu;
            for (int s2 = 0; s2 < S; s2++) {
                if (counts && rdme) counts[o * S + s2] = (int32_t)b.u0[(size_t)i * S + s2];
                if (chem && sc->enable_pde) chem[o * S + s2] = p.C[s2];
            }
        }
        oi++;
    };
    for (sys->current_step = 0; sys->current_step < sys->nt; sys->current_step++) {
        buildKDTree(sys);
        if (sys->current_step >= next_output && oi < sc->num_outputs) {
            snap();
            next_output = get_next_output(sys);
        }
        for (unsigned sub = 0; sub < 3; sub++)
            for (auto &p : sys->particles) take_step(&p, sys, sys->current_step, sub);
        if (rdme) simulate_rdme(sys, sys->current_step);
    }
    while (oi < sc->num_outputs) snap();
    if (chdir(cwd) != 0) return SP_E_INVALID;
    return SP_OK;
}

/*
 * CPU baselines of the moving domain: the engine loop of spref_coupled
 * (with_rdme: species on; else the flow alone) over steps [0, nt), timing
 * steps [timed_from, nt) only (the set-up and the first steps excluded).
 * counters: (reactions, diffusions) in the timed steps; *seconds: their wall
 * time (steady clock).
 */
int spref_moving_bench(const sp_scenario *sc, const uint32_t *u0, uint64_t seed, int32_t with_rdme,
                       int32_t timed_from, int64_t *counters, double *seconds) {
    Built b;
    const int rdme = with_rdme && sc->num_species > 0;
    int rc = build(sc, b, rdme);
    if (rc) return rc;
    ParticleSystem *sys = b.sys;
    if (sys->static_domain) return SP_E_UNSUPPORTED;
    if (timed_from < 0 || timed_from >= (int)sc->num_steps) return SP_E_INVALID;
    const int S = sc->num_species, N = sc->num_particles;
    if (rdme) {
        b.u0.assign(u0, u0 + (size_t)N * S);
        rng = std::mt19937_64(seed);
        initialize_rdme(sys, b.irN.data(), b.jcN.data(), b.prN.data(), b.irG.data(),
                        b.jcG.data(), b.u0.data());
    }
    long long r0 = 0, d0 = 0;
    auto t0 = std::chrono::steady_clock::now();
    for (sys->current_step = 0; sys->current_step < sys->nt; sys->current_step++) {
        if ((int)sys->current_step == timed_from) {
            r0 = sys->total_reactions;
            d0 = sys->total_diffusion;
            t0 = std::chrono::steady_clock::now();
        }
        buildKDTree(sys);
        for (unsigned sub = 0; sub < 3; sub++)
            for (auto &p : sys->particles) take_step(&p, sys, sys->current_step, sub);
        if (rdme) simulate_rdme(sys, sys->current_step);
    }
    const auto t1 = std::chrono::steady_clock::now();
    counters[0] = sys->total_reactions - r0;
    counters[1] = sys->total_diffusion - d0;
    *seconds = std::chrono::duration<double>(t1 - t0).count();
    return SP_OK;
}

/*
 * SDPD flow without species: nsteps engine steps (substeps 0,1,2 over all
 * particles in order, single-threaded).  Writes final x[N*3], v[N*3],
 * rho[N], and the last neighbour counts.
 */
int spref_sdpd(const sp_scenario *sc, int32_t nsteps, double *x, double *v, double *rho) {
    Built b;
    int rc = build(sc, b, 0);
    if (rc) return rc;
    ParticleSystem *sys = b.sys;
    for (sys->current_step = 0; sys->current_step < (unsigned)nsteps; sys->current_step++) {
        buildKDTree(sys);
        for (unsigned sub = 0; sub < 3; sub++)
            for (auto &p : sys->particles) take_step(&p, sys, sys->current_step, sub);
    }
    for (size_t i = 0; i < sys->particles.size(); i++) {
        const Particle &p = sys->particles[i];
        for (int d = 0; d < 3; d++) {
            x[3 * i + d] = p.x[d];
            v[3 * i + d] = p.v[d];
        }
        rho[i] = p.rho;
    }
    return SP_OK;
}

}  // extern "C"
