// engine.cu — the C ABI of libspgpu (include/spgpu.h): handle lifecycle,
// device set-up of model instances, and the host loop of an ensemble run.
//
// sp_create  = Solver.compile() + engine set-up (solver.py:443-507,
//              propensity_file_template.cpp:101-142)
// sp_run     = Solver.run()'s trajectory loop (solver.py:547-605) + the
//              engine step loop run_simulation (simulate_threads.cpp:171-312)
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "chem.cuh"
#include "common.cuh"
#include "neighbors.cuh"
#include "sdpd.cuh"

namespace spg {
void launch_nsm_init(NsmTraj* trajs, const NsmInstance* insts, int ntraj, int max_leaf,
                     int max_levels, const uint32_t* const* u0, bool build_queue,
                     cudaStream_t st);
void launch_nsm_rebuild(NsmTraj* trajs, const NsmInstance* insts, int ntraj, int max_leaf,
                        int max_levels, double t0, uint32_t build_index, int variant,
                        cudaStream_t st);
int nsm_warp_smem(const NsmInstance& d, bool with_state);
void launch_nsm_advance(bool ref, bool smem_state, int variant, int warp_smem, int wpb,
                        NsmTraj* trajs, const NsmInstance* insts, int ntraj, int step_end,
                        double dt, long long budget, long long max_ns, int* work, int num_sms,
                        const int* tlist, cudaStream_t st);
int nsm_batch_smem(const NsmInstance& d);
int nsm_batchw_smem(const NsmInstance& d, int W);
void launch_nsm_batchw(bool ref, int variant, int warps, int smem_bytes, NsmTraj* trajs,
                       const NsmInstance* insts, int ntraj, int step_end, double dt,
                       long long budget, long long max_ns, int* work, int num_sms,
                       const int* tlist, cudaStream_t st);
void launch_nsm_batch(bool ref, int variant, int warp_smem, NsmTraj* trajs,
                      const NsmInstance* insts, int ntraj, int step_end, double dt,
                      long long budget, long long max_ns, int* work, int num_sms,
                      const int* tlist, cudaStream_t st);
void launch_nsm_snapshot(const NsmTraj* trajs, const NsmInstance* insts, int ntraj,
                         int32_t* counts, const long long* count_off, long long* moments,
                         const long long* mom_off, int out_index, cudaStream_t st);
}  // namespace spg

using namespace spg;

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t n = 0;
};

struct Instance {
    int N = 0, S = 0, R = 0, T = 0, K = 0, dim = 0;
    bool is_static = true;
    double h = 0, rho0 = 0, c0 = 0, P0 = 0, g[3] = {0, 0, 0};
    std::vector<double> x_host;
    // device arrays
    double *x = nullptr, *mass = nullptr, *rho = nullptr, *nu = nullptr;
    float *vol = nullptr, *ivol = nullptr;
    int *type = nullptr;
    uint8_t* fixed = nullptr;
    int *nbr_cnt = nullptr, *nbr_idx = nullptr;
    double *nbr_dist = nullptr, *nbr_dwdr = nullptr, *nbr_dij = nullptr;
    float *cdf = nullptr, *ddiag = nullptr, *rate = nullptr;
    int2* cdfj = nullptr;
    double* diffusion = nullptr;
    int *kind = nullptr, *reac = nullptr, *jcN = nullptr, *irN = nullptr, *prN = nullptr;
    uint8_t* allowed = nullptr;
    int *code = nullptr, *code_off = nullptr;
    double *consts = nullptr, *data = nullptr;
    int num_data = 0;
    bool has_custom = false;
    uint32_t* u0 = nullptr;   // device copy for the current run
    NsmInstance desc{};
    SdpdState* sdpd = nullptr;
    // deterministic chemistry (enable_pde)
    bool pde = false;
    ChemDev chem{};
};

}  // namespace

// One event kernel and its launch shape over a set of trajectories.
struct KernelGroup {
    bool batch = false, smem_state = false;
    int variant = 0, warp_smem = 0, wpb = 1;
    int warps = 1;             // batch kernel: warps per trajectory (1, 2 or 4)
    std::vector<int> list;     // trajectories, in launch order
    int* d_list = nullptr;     // device copy, or nullptr for 0..ntraj-1
};

// Warps-per-trajectory tuner of a batch group: the first output intervals
// run with 4, 2 and 1 warps per trajectory in turn; the width with the
// highest events/ms is kept.  Every width gives the same events, so the
// choice changes speed only.
struct WarpTuner {
    bool on = false;
    int stage = 0;
    double rate[3] = {0, 0, 0};
    static constexpr int widths[3] = {4, 2, 1};
};

struct RunState {
    bool active = false;
    sp_run_args args{};
    sp_outputs out{};
    std::vector<int> inst;
    std::vector<void*> tmp;
    std::chrono::steady_clock::time_point wall0;
    bool want_counts = false, want_mom = false;
    int next_out = 0, result = SP_OK;
    // kernel groups, each on its own stream: with the default policy the
    // batch trajectories and the small domains (sequential kernel)
    KernelGroup grp[2];
    int ngroups = 1;
    WarpTuner tune;
    long long ctot = 0, mtot = 0;
    int32_t* d_counts = nullptr;
    long long *d_mom = nullptr, *d_coff = nullptr, *d_moff = nullptr;
    // moving domain with species: one flow (instance cinst) shared by every
    // trajectory, stepped here; particle outputs of that instance
    bool coupled = false, want_part = false;
    bool chem = false, want_chem = false;   // some instance has enable_pde
    int chem_step = 0;                      // static domains: chemistry steps taken
    double* d_chem = nullptr;               // chemistry outputs
    long long chem_tot = 0;
    std::vector<long long> chem_off;        // per instance, in doubles
    int cinst = -1, step = 0, max_leaf = 0, max_levels = 0;
    int rebuild_variant = 0;   // register-resident network of the per-step queue rebuild
    long long poff = 0, ptot = 0;   // offset of cinst / total, in particles x outputs
    double *d_px = nullptr, *d_pv = nullptr, *d_prho = nullptr;
};

struct sp_handle {
    int device = 0;
    int num_sms = 0;
    cudaStream_t st = nullptr, st2 = nullptr;   // st2: the second kernel group
    cudaEvent_t e0 = nullptr, e1 = nullptr, ea = nullptr, eb = nullptr, fork = nullptr,
                join = nullptr;
    sp_options opt{};
    std::vector<Instance> inst;
    std::vector<void*> allocs;
    NsmInstance* d_insts = nullptr;
    double dt = 0;
    int num_steps = 0;
    std::vector<int> output_steps;
    // run state
    int traj_cap = 0;
    size_t traj_bytes = 0;
    void* traj_mem = nullptr;
    NsmTraj* d_trajs = nullptr;
    std::vector<NsmTraj> h_trajs;
    int* d_work = nullptr;
    std::string err;
    double last_ms = 0, adv_ms = 0;
    long long last_launches = 0, launches = 0;
    int last_kernel = SP_KERNEL_NONE;
    RunState run;
};

int spg_set_cuda_error(sp_handle* h, cudaError_t e, const char* what, const char* file, int line) {
    if (h) {
        char buf[512];
        snprintf(buf, sizeof buf, "CUDA error %s (%s) at %s:%d: %s", cudaGetErrorName(e), what,
                 file, line, cudaGetErrorString(e));
        h->err = buf;
    }
    return e == cudaErrorMemoryAllocation ? SP_E_NOMEM : SP_E_CUDA;
}

static int fail(sp_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    return code;
}

template <typename T>
static int dev_upload(sp_handle* h, T** dst, const T* src, size_t n) {
    *dst = nullptr;
    if (n == 0) return SP_OK;
    SP_CUDA_TRY(cudaMalloc((void**)dst, sizeof(T) * n));
    h->allocs.push_back(*dst);
    if (src) SP_CUDA_TRY(cudaMemcpyAsync(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice, h->st));
    return SP_OK;
}

template <typename T>
static int dev_alloc(sp_handle* h, T** dst, size_t n) {
    return dev_upload<T>(h, dst, nullptr, n);
}

// A custom propensity program must stay inside its reaction's slice, take
// operands in range, never underflow, stay within SP_PROG_MAX_STACK values and
// end at SP_OP_END with one value: then the kernels' interpreter cannot read
// or write out of bounds.  Returns nullptr, or what is wrong.
static const char* check_program_in(const sp_scenario& s, const int32_t* code,
                                    const int64_t* offs, int num_consts, int r) {
    const int64_t b = offs[r], e = offs[r + 1];
    if (b < 0 || e < b || e > offs[s.num_reactions]) return "program offsets out of order";
    if (b == e) return "empty program";
    int d = 0;
    for (int64_t pc = b; pc < e;) {
        const int op = code[pc];
        const int64_t need = (op == SP_OP_CONST || op == SP_OP_X || op == SP_OP_DATA ||
                              op == SP_OP_POWI) ? 2 : 1;
        if (pc + need > e) return "operand past the end of the program";
        const int a = need == 2 ? code[pc + 1] : 0;
        if (op == SP_OP_END) return d == 1 ? nullptr : "program does not leave one value";
        if (op == SP_OP_CONST) {
            if (a < 0 || a >= num_consts) return "constant index out of range";
            d++;
        } else if (op == SP_OP_X) {
            if (a < 0 || a >= s.num_species) return "species index out of range";
            d++;
        } else if (op == SP_OP_DATA) {
            if (a < 0 || a >= s.num_data_fn || !s.data_fn) return "data function index out of range";
            d++;
        } else if (op == SP_OP_VOL || op == SP_OP_T || op == SP_OP_TYPE) {
            d++;
        } else if (op == SP_OP_POWI) {
            if (a < -64 || a > 64) return "integer power out of range";
            if (d < 1) return "stack underflow";
        } else if (op == SP_OP_NEG || op == SP_OP_NOT || (op >= SP_OP_EXP && op <= SP_OP_CEIL)) {
            if (d < 1) return "stack underflow";
        } else if ((op >= SP_OP_ADD && op <= SP_OP_POW) || (op >= SP_OP_LT && op <= SP_OP_OR)) {
            if (d < 2) return "stack underflow";
            d--;
        } else {
            return "unknown opcode";
        }
        if (d > SP_PROG_MAX_STACK) return "program needs more than 16 stack values";
        pc += need;
    }
    return "program without END";
}

static const char* check_program(const sp_scenario& s, int r) {
    return check_program_in(s, s.rxn_code, s.rxn_code_off, s.num_consts, r);
}

static int validate(sp_handle* h, const sp_scenario& s, int i) {
    char b[256];
#define REQ(cond, msg)                                           \
    if (!(cond)) {                                               \
        snprintf(b, sizeof b, "scenario %d: %s", i, msg);        \
        return fail(h, SP_E_INVALID, b);                         \
    }
    REQ(s.dimension >= 1 && s.dimension <= 3, "dimension must be 1, 2 or 3");
    REQ(s.num_particles >= 1, "num_particles must be >= 1");
    REQ(s.x && s.type && s.mass && s.rho && s.nu && s.fixed, "particle arrays must be set");
    REQ(s.num_types >= 1, "num_types must be >= 1");
    REQ(s.num_species >= 0 && s.num_species <= 32, "num_species must be in 0..32");
    REQ(s.num_reactions >= 0 && s.num_reactions <= 1024, "num_reactions must be in 0..1024");
    REQ(s.h > 0, "h (basis function width) can not be zero");
    REQ(s.dt > 0 && s.num_steps >= 0, "dt must be > 0");
    REQ(s.num_outputs >= 1 && s.output_steps, "output_steps must be set");
    for (int k = 0; k < s.num_outputs; k++) {
        REQ(s.output_steps[k] >= 0 && s.output_steps[k] <= s.num_steps, "output step out of range");
        REQ(k == 0 || s.output_steps[k] > s.output_steps[k - 1], "output steps must ascend");
    }
    for (int p = 0; p < s.num_particles; p++) {
        REQ(s.type[p] >= 1 && s.type[p] <= s.num_types, "particle type out of 1..num_types");
        REQ(s.rho[p] != 0.0, "Rho must be a positive value");
    }
    if (s.num_species > 0) {
        REQ(s.diffusion, "diffusion matrix must be set");
        if (s.num_reactions > 0) {
            REQ(s.rxn_rate && s.rxn_kind && s.rxn_reactants && s.jcN && s.irN && s.prN,
                "reaction tables must be set");
            REQ(s.jcN[0] == 0, "jcN[0] must be 0");
        }
        for (int r = 0; r < s.num_reactions; r++) {
            const int k = s.rxn_kind[r];
            REQ(k >= SP_RXN_ZERO && k <= SP_RXN_CUSTOM, "unknown reaction kind");
            if (k == SP_RXN_CUSTOM) {
                REQ(s.rxn_code && s.rxn_code_off && (s.rxn_consts || s.num_consts == 0),
                    "custom propensity programs must be set");
                const char* why = check_program(s, r);
                if (why) {
                    snprintf(b, sizeof b, "scenario %d: reaction %d: %s", i, r, why);
                    return fail(h, SP_E_INVALID, b);
                }
            } else {
                const int a = s.rxn_reactants[2 * r], bb = s.rxn_reactants[2 * r + 1];
                REQ(k == SP_RXN_ZERO || (a >= 0 && a < s.num_species), "reactant index out of range");
                REQ(k != SP_RXN_SECOND || (bb >= 0 && bb < s.num_species),
                    "second reactant out of range");
            }
            REQ(s.jcN[r + 1] >= s.jcN[r], "jcN must be non-decreasing");
            for (int64_t q = s.jcN[r]; q < s.jcN[r + 1]; q++)
                REQ(s.irN[q] >= 0 && s.irN[q] < s.num_species, "irN out of range");
        }
    }
    if (s.enable_pde && s.num_species > 0) {
        REQ(s.num_reactions == 0 || (s.ode_code && s.ode_code_off && s.ode_consts),
            "enable_pde needs the reactions' ODE rate programs");
        for (int r = 0; r < s.num_reactions; r++) {
            const char* why = check_program_in(s, s.ode_code, s.ode_code_off, s.num_ode_consts, r);
            if (why) {
                snprintf(b, sizeof b, "scenario %d: ODE rate of reaction %d: %s", i, r, why);
                return fail(h, SP_E_INVALID, b);
            }
        }
    }
    REQ(s.num_bcs >= 0, "num_bcs must be >= 0");
    if (s.num_bcs > 0) {
        REQ(s.bc_box && s.bc_type && s.bc_target && s.bc_value, "boundary condition arrays must be set");
        for (int q = 0; q < s.num_bcs; q++)
            REQ(s.bc_target[q] >= SP_BC_V && s.bc_target[q] < SP_BC_C + s.num_species,
                "boundary condition target out of range");
    }
#undef REQ
    return SP_OK;
}

static void tree_layout(NsmInstance& d, int N) {
    d.leaf_stride = (N + 31) / 32 * 32;
    int size = d.leaf_stride, l = 0, off = 0;
    d.level_size[0] = N;
    d.level_off[0] = 0;
    do {
        size = (size + 31) / 32;
        l++;
        d.level_size[l] = size;
        d.level_off[l] = off;
        off += size;
    } while (size > 1 && l < kMaxLevels);
    d.levels = l;
    d.num_nodes = off;
}

static int setup_instance(sp_handle* h, const sp_scenario& s, Instance& I) {
    I.N = s.num_particles;
    I.S = s.num_species;
    I.R = s.num_reactions;
    I.T = s.num_types;
    I.dim = s.dimension;
    I.h = s.h;
    I.rho0 = s.rho0;
    I.c0 = s.c0;
    I.P0 = s.P0;
    for (int d = 0; d < 3; d++) I.g[d] = s.gravity[d];
    I.is_static = s.static_domain != 0;
    const int N = I.N;
    I.x_host.assign(s.x, s.x + 3 * (size_t)N);
    int rc;
    if ((rc = dev_upload(h, &I.x, s.x, 3 * (size_t)N))) return rc;
    if ((rc = dev_upload(h, &I.type, s.type, N))) return rc;
    if ((rc = dev_upload(h, &I.mass, s.mass, N))) return rc;
    if ((rc = dev_upload(h, &I.rho, s.rho, N))) return rc;
    if ((rc = dev_upload(h, &I.nu, s.nu, N))) return rc;
    if ((rc = dev_upload(h, &I.fixed, s.fixed, N))) return rc;
    std::vector<float> vol(N), ivol(N);
    for (int p = 0; p < N; p++) {
        vol[p] = (float)(s.mass[p] / s.rho[p]);   // simulate_rdme.cpp:123
        ivol[p] = (float)(s.rho[p] / s.mass[p]);
    }
    if ((rc = dev_upload(h, &I.vol, vol.data(), N))) return rc;
    if ((rc = dev_upload(h, &I.ivol, ivol.data(), N))) return rc;
    // reaction tables
    const int R = I.R, S = I.S, T = I.T;
    std::vector<int> jc(R + 1, 0), ir, pr;
    if (R > 0) {
        for (int r = 0; r <= R; r++) jc[r] = (int)s.jcN[r];
        ir.assign(s.irN, s.irN + s.jcN[R]);
        pr.assign(s.prN, s.prN + s.jcN[R]);
        std::vector<float> rate(R);
        for (int r = 0; r < R; r++) rate[r] = (float)s.rxn_rate[r];
        if ((rc = dev_upload(h, &I.rate, rate.data(), R))) return rc;
        if ((rc = dev_upload(h, &I.kind, s.rxn_kind, R))) return rc;
        if ((rc = dev_upload(h, &I.reac, s.rxn_reactants, 2 * (size_t)R))) return rc;
        if (s.rxn_allowed && (rc = dev_upload(h, &I.allowed, s.rxn_allowed, (size_t)R * (T + 1))))
            return rc;
    }
    if ((rc = dev_upload(h, &I.jcN, jc.data(), jc.size()))) return rc;
    if (!ir.empty()) {
        if ((rc = dev_upload(h, &I.irN, ir.data(), ir.size()))) return rc;
        if ((rc = dev_upload(h, &I.prN, pr.data(), pr.size()))) return rc;
    }
    if (S > 0 && (rc = dev_upload(h, &I.diffusion, s.diffusion, (size_t)S * T))) return rc;
    // custom propensity programs (checked by validate) and data functions
    for (int r = 0; r < R; r++) I.has_custom |= s.rxn_kind[r] == SP_RXN_CUSTOM;
    if (I.has_custom) {
        const int64_t len = s.rxn_code_off[R];
        std::vector<int> off(R + 1);
        for (int r = 0; r <= R; r++) off[r] = (int)s.rxn_code_off[r];
        if ((rc = dev_upload(h, &I.code, s.rxn_code, (size_t)len))) return rc;
        if ((rc = dev_upload(h, &I.code_off, off.data(), off.size()))) return rc;
        const double zero = 0.0;
        if ((rc = dev_upload(h, &I.consts, s.num_consts > 0 ? s.rxn_consts : &zero,
                             (size_t)(s.num_consts > 0 ? s.num_consts : 1))))
            return rc;
    }
    if (s.num_data_fn > 0 && s.data_fn) {
        I.num_data = s.num_data_fn;
        if ((rc = dev_upload(h, &I.data, s.data_fn, (size_t)s.num_data_fn * N))) return rc;
    }

    if (I.is_static) {
        // neighbour lists once (take_step1 at step 0, simulate.cpp:62-64)
        CellGrid g = make_grid(s.x, N, I.dim, I.h);
        int *cell, *hist, *start, *fill, *order, *flag;
        if ((rc = dev_alloc(h, &cell, N))) return rc;
        if ((rc = dev_alloc(h, &hist, g.ncell))) return rc;
        if ((rc = dev_alloc(h, &start, (size_t)g.ncell + 1))) return rc;
        if ((rc = dev_alloc(h, &fill, g.ncell))) return rc;
        if ((rc = dev_alloc(h, &order, N))) return rc;
        if ((rc = dev_alloc(h, &flag, 1))) return rc;
        int kmax = 32;
        for (;;) {
            int *cnt, *idx;
            double *dist, *dw, *dij;
            if ((rc = dev_alloc(h, &cnt, N))) return rc;
            if ((rc = dev_alloc(h, &idx, (size_t)N * kmax))) return rc;
            if ((rc = dev_alloc(h, &dist, (size_t)N * kmax))) return rc;
            if ((rc = dev_alloc(h, &dw, (size_t)N * kmax))) return rc;
            if ((rc = dev_alloc(h, &dij, (size_t)N * kmax))) return rc;
            const int over = run_neighbor_search(I.x, I.x, N, g, I.h, I.mass, I.rho, kmax, cnt, idx,
                                                 dist, dw, dij, cell, hist, start, fill, order,
                                                 flag, h->st);
            SP_CUDA_TRY(cudaGetLastError());
            if (!over) {
                I.K = kmax;
                I.nbr_cnt = cnt;
                I.nbr_idx = idx;
                I.nbr_dist = dist;
                I.nbr_dwdr = dw;
                I.nbr_dij = dij;
                break;
            }
            if (kmax >= 256) return fail(h, SP_E_UNSUPPORTED, "more than 256 neighbours within h");
            kmax *= 2;
        }
        if (S > 0) {
            if ((rc = dev_alloc(h, &I.ddiag, (size_t)N * S))) return rc;
            if ((rc = dev_alloc(h, &I.cdf, (size_t)N * S * I.K))) return rc;
            if ((rc = dev_alloc(h, &I.cdfj, (size_t)N * S * I.K))) return rc;
            launch_diffusion_tables(N, S, T, I.K, I.type, I.nbr_cnt, I.nbr_idx, I.nbr_dij,
                                    I.diffusion, I.ddiag, I.cdf, I.cdfj, h->st);
            SP_CUDA_TRY(cudaGetLastError());
        }
    } else {
        I.sdpd = sdpd_create(s, h->opt.sdpd_precision, h->opt.sdpd_self_pair, h->st, &h->err);
        if (!I.sdpd) return SP_E_CUDA;
        if (S > 0) {
            // species on a moving domain: the flow's force-pass lists carry
            // D_ij and feed the per-step diffusion tables
            if ((rc = sdpd_enable_dij(I.sdpd, &h->err))) return rc;
            const SdpdLists L = sdpd_lists(I.sdpd);
            I.K = L.kcap;
            I.nbr_cnt = L.count;
            I.nbr_idx = L.idx;
            if ((rc = dev_alloc(h, &I.ddiag, (size_t)N * S))) return rc;
            if ((rc = dev_alloc(h, &I.cdf, (size_t)N * S * I.K))) return rc;
            if ((rc = dev_alloc(h, &I.cdfj, (size_t)N * S * I.K))) return rc;
            SP_CUDA_TRY(cudaMemsetAsync(I.ddiag, 0, sizeof(float) * N * S, h->st));
            SP_CUDA_TRY(cudaMemsetAsync(I.cdf, 0, sizeof(float) * N * S * I.K, h->st));
            SP_CUDA_TRY(cudaMemsetAsync(I.cdfj, 0, sizeof(int2) * N * S * I.K, h->st));
        }
    }
    NsmInstance& d = I.desc;
    d.N = N;
    d.S = S;
    d.R = R;
    d.T = T;
    d.K = I.K;
    tree_layout(d, N);
    d.type = I.type;
    d.vol = I.vol;
    d.ivol = I.ivol;
    d.nbr_cnt = I.nbr_cnt;
    d.nbr_idx = I.nbr_idx;
    d.cdf = I.cdf;
    d.cdfj = I.cdfj;
    d.ddiag = I.ddiag;
    d.rate = I.rate;
    d.kind = I.kind;
    d.reac = I.reac;
    d.allowed = I.allowed;
    d.jcN = I.jcN;
    d.irN = I.irN;
    d.prN = I.prN;
    d.code = I.code;
    d.code_off = I.code_off;
    d.consts = I.consts;
    d.data = I.data;
    d.num_data = I.num_data;
    d.has_custom = I.has_custom ? 1 : 0;
    d.has_source = 0;
    for (int r = 0; r < R; r++)
        if (s.rxn_kind[r] == SP_RXN_ZERO || s.rxn_kind[r] == SP_RXN_CUSTOM) d.has_source = 1;
    if (s.enable_pde && S > 0) {
        ChemDev& D = I.chem;
        I.pde = true;
        D.N = N;
        D.S = S;
        D.R = R;
        D.T = T;
        D.dt = s.dt;
        D.h = s.h;
        if ((rc = dev_alloc(h, &D.C, (size_t)N * S))) return rc;
        if ((rc = dev_alloc(h, &D.Q, (size_t)N * S))) return rc;
        D.type = I.type;
        D.diffusion = I.diffusion;
        D.allowed = I.allowed;
        D.data = I.data;
        if (R > 0) {
            std::vector<int> dense((size_t)S * R, 0), off(R + 1);
            for (int r = 0; r < R; r++)
                for (int64_t q = s.jcN[r]; q < s.jcN[r + 1]; q++)
                    dense[(size_t)s.irN[q] * R + r] += s.prN[q];
            int* st = nullptr;
            if ((rc = dev_upload(h, &st, dense.data(), dense.size()))) return rc;
            D.stoich = st;
            const int64_t len = s.ode_code_off[R];
            for (int r = 0; r <= R; r++) off[r] = (int)s.ode_code_off[r];
            int *code = nullptr, *co = nullptr;
            double* cs = nullptr;
            if ((rc = dev_upload(h, &code, s.ode_code, (size_t)len))) return rc;
            if ((rc = dev_upload(h, &co, off.data(), off.size()))) return rc;
            const double zero = 0.0;
            if ((rc = dev_upload(h, &cs, s.num_ode_consts > 0 ? s.ode_consts : &zero,
                                 (size_t)(s.num_ode_consts > 0 ? s.num_ode_consts : 1))))
                return rc;
            D.code = code;
            D.code_off = co;
            D.consts = cs;
        }
        if (s.num_bcs > 0) {
            const int nb = s.num_bcs;
            double *box = nullptr, *val = nullptr;
            int *ty = nullptr, *tg = nullptr;
            if ((rc = dev_upload(h, &box, s.bc_box, 6 * (size_t)nb))) return rc;
            if ((rc = dev_upload(h, &val, s.bc_value, 3 * (size_t)nb))) return rc;
            if ((rc = dev_upload(h, &ty, s.bc_type, (size_t)nb))) return rc;
            if ((rc = dev_upload(h, &tg, s.bc_target, (size_t)nb))) return rc;
            D.nbc = nb;
            D.bc_box = box;
            D.bc_value = val;
            D.bc_type = ty;
            D.bc_target = tg;
        }
    }
    return SP_OK;
}

extern "C" {

int sp_abi_version(void) { return SP_ABI_VERSION; }

int sp_create(const sp_scenario* scenarios, int32_t num_scenarios, const sp_options* opts,
              sp_handle** out) {
    if (!out) return SP_E_INVALID;
    *out = nullptr;
    if (!scenarios || num_scenarios < 1) return SP_E_INVALID;
    sp_handle* h = new sp_handle();
    if (opts) h->opt = *opts;
    *out = h;
    h->device = h->opt.device;
    // arguments are checked before any device call
    for (int i = 0; i < num_scenarios; i++) {
        int rc = validate(h, scenarios[i], i);
        if (rc) return rc;
    }
    const sp_scenario& s0 = scenarios[0];
    for (int i = 1; i < num_scenarios; i++) {
        const sp_scenario& s = scenarios[i];
        if (s.dt != s0.dt || s.num_steps != s0.num_steps || s.num_outputs != s0.num_outputs ||
            !std::equal(s.output_steps, s.output_steps + s.num_outputs, s0.output_steps))
            return fail(h, SP_E_INVALID, "all instances of one handle need the same time span");
    }
    SP_CUDA_TRY(cudaSetDevice(h->device));
    SP_CUDA_TRY(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device));
    SP_CUDA_TRY(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
    SP_CUDA_TRY(cudaEventCreate(&h->e0));
    SP_CUDA_TRY(cudaEventCreate(&h->e1));
    SP_CUDA_TRY(cudaEventCreate(&h->ea));
    SP_CUDA_TRY(cudaEventCreate(&h->eb));
    SP_CUDA_TRY(cudaStreamCreateWithFlags(&h->st2, cudaStreamNonBlocking));
    SP_CUDA_TRY(cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming));
    SP_CUDA_TRY(cudaEventCreateWithFlags(&h->join, cudaEventDisableTiming));
    h->dt = s0.dt;
    h->num_steps = s0.num_steps;
    h->output_steps.assign(s0.output_steps, s0.output_steps + s0.num_outputs);
    h->inst.resize(num_scenarios);
    std::vector<NsmInstance> descs(num_scenarios);
    for (int i = 0; i < num_scenarios; i++) {
        int rc = setup_instance(h, scenarios[i], h->inst[i]);
        if (rc) return rc;
        descs[i] = h->inst[i].desc;
    }
    int rc = dev_upload(h, &h->d_insts, descs.data(), descs.size());
    if (rc) return rc;
    if ((rc = dev_alloc(h, &h->d_work, 2))) return rc;
    SP_CUDA_TRY(cudaStreamSynchronize(h->st));
    return SP_OK;
}

static int ensure_traj(sp_handle* h, int ntraj, const int* inst) {
    size_t bytes = sizeof(NsmTraj) * (size_t)ntraj;
    std::vector<size_t> off(ntraj);
    auto align = [](size_t b) { return (b + 255) / 256 * 256; };
    bytes = align(bytes);
    for (int j = 0; j < ntraj; j++) {
        const NsmInstance& d = h->inst[inst[j]].desc;
        off[j] = bytes;
        bytes += align(sizeof(int32_t) * (size_t)d.N * d.S);
        bytes += align(sizeof(long long) * (size_t)d.leaf_stride);
        bytes += align(sizeof(long long) * (size_t)d.num_nodes);
        bytes += align(sizeof(int32_t) * (size_t)d.num_nodes);
        bytes += align(sizeof(long long) * (size_t)d.level_size[1]);
    }
    if (bytes > h->traj_bytes) {
        if (h->traj_mem) cudaFree(h->traj_mem);
        h->traj_mem = nullptr;
        h->traj_bytes = 0;
        SP_CUDA_TRY(cudaMalloc(&h->traj_mem, bytes));
        h->traj_bytes = bytes;
    }
    char* base = (char*)h->traj_mem;
    h->d_trajs = (NsmTraj*)base;
    h->h_trajs.assign(ntraj, NsmTraj{});
    for (int j = 0; j < ntraj; j++) {
        const NsmInstance& d = h->inst[inst[j]].desc;
        NsmTraj& T = h->h_trajs[j];
        T.inst = inst[j];
        char* p = base + off[j];
        T.x = (int32_t*)p;
        p += align(sizeof(int32_t) * (size_t)d.N * d.S);
        T.leaf = (long long*)p;
        p += align(sizeof(long long) * (size_t)d.leaf_stride);
        T.node_t = (long long*)p;
        p += align(sizeof(long long) * (size_t)d.num_nodes);
        T.node_i = (int32_t*)p;
        p += align(sizeof(int32_t) * (size_t)d.num_nodes);
        T.node_t2 = (long long*)p;
    }
    return SP_OK;
}

// ---------------------------------------------------------------------------
// ensemble runs: start (upload, queue build, output 0), continue (advance
// through further outputs), finish (copy results to the caller)
// ---------------------------------------------------------------------------
static void run_release(sp_handle* h) {
    RunState& R = h->run;
    for (void* p : R.tmp) cudaFree(p);
    R.tmp.clear();
    R.active = false;
}

// register-resident network variant for the trajectories `js` (0 = generic)
static int net_variant(sp_handle* h, const std::vector<int>& js, const std::vector<int>& inst) {
    int minS = 1 << 30, minR = 1 << 30, maxS = 0, maxR = 0, maxT = 0;
    for (int j : js) {
        const Instance& I = h->inst[inst[j]];
        if (I.has_custom) return 0;   // programs run in the generic kernel only
        minS = std::min(minS, I.S);
        minR = std::min(minR, I.R);
        maxS = std::max(maxS, I.S);
        maxR = std::max(maxR, I.R);
        maxT = std::max(maxT, I.T);
    }
    if (h->opt.nsm_variant == 1) return 0;   // the generic warp kernel, forced
    if (maxT < 64 && minS == maxS && minR == maxR && maxS == 1 && maxR == 2) return 3;
    if (maxT < 64 && minS == maxS && minR == maxR && maxS == 3 && maxR == 4) return 4;
    if (maxT < 64 && maxS <= 4 && maxR <= 8) return 1;
    if (maxT < 64 && maxS <= 8 && maxR <= 16) return 2;
    return 0;
}

// batch width of group G (falls back to fewer warps when shared memory is short)
static void set_warps(sp_handle* h, const RunState& R, KernelGroup& G, int W) {
    for (; W > 1; W >>= 1) {
        int wb = 0;
        for (int j : G.list) wb = std::max(wb, nsm_batchw_smem(h->inst[R.inst[j]].desc, W));
        if (wb <= 200 * 1024) {
            G.warps = W;
            G.warp_smem = wb;
            return;
        }
    }
    int wb = 0;
    for (int j : G.list) wb = std::max(wb, nsm_batch_smem(h->inst[R.inst[j]].desc));
    G.warps = 1;
    G.warp_smem = wb;
}

static int kernel_kind(const RunState& R) {
    return R.ngroups == 2 ? SP_KERNEL_MIXED
         : R.grp[0].batch && R.grp[0].warps == 2 ? SP_KERNEL_BATCH_W2
         : R.grp[0].batch && R.grp[0].warps == 4 ? SP_KERNEL_BATCH_W4
         : R.grp[0].batch ? SP_KERNEL_BATCH
         : R.grp[0].variant != 0 ? SP_KERNEL_SEQUENTIAL : SP_KERNEL_GENERIC;
}

// kernel and launch shape for the trajectories `js`
static int choose_group(sp_handle* h, const RunState& R, const std::vector<int>& js,
                        bool want_batch, KernelGroup& G) {
    int state_bytes = 0, tree_bytes = 0, batch_bytes = 0;
    for (int j : js) {
        const NsmInstance& d = h->inst[R.inst[j]].desc;
        state_bytes = std::max(state_bytes, nsm_warp_smem(d, true));
        tree_bytes = std::max(tree_bytes, nsm_warp_smem(d, false));
        batch_bytes = std::max(batch_bytes, nsm_batch_smem(d));
    }
    G.list = js;
    // shared-memory policy: whole trajectory state when it fits in 48 KB per
    // warp, else the tree only (levels >= 1, 12 bytes per node)
    G.smem_state = state_bytes <= 48 * 1024;
    G.warp_smem = G.smem_state ? state_bytes : tree_bytes;
    if (G.warp_smem > 200 * 1024)
        return fail(h, SP_E_UNSUPPORTED, "domain too large for the shared-memory event queue");
    G.wpb = G.warp_smem <= 24 * 1024 ? 4 : G.warp_smem <= 48 * 1024 ? 2 : 1;
    G.variant = net_variant(h, js, R.inst);
    // speculative batches need a register-resident network
    G.batch = want_batch && G.variant != 0 && batch_bytes <= 200 * 1024;
    if (G.batch) G.warp_smem = batch_bytes;
    // warps per trajectory: forced by nsm_variant 4 (2 warps) or 5 (4 warps);
    // by default 4 while the trajectories fit about three CTAs per SM, 2 up to
    // six, else 1 (the tuner refines this on long runs)
    const int n = (int)js.size();
    const int W = h->opt.nsm_variant == 4 ? 2 : h->opt.nsm_variant == 5 ? 4
                : h->opt.nsm_variant != 0 ? 1
                : n <= 3 * h->num_sms ? 4 : n <= 6 * h->num_sms ? 2 : 1;
    if (G.batch) set_warps(h, R, G, W);
    return SP_OK;
}

// one launch of every kernel group, to step_end; group 1 runs on st2
static void launch_groups(sp_handle* h, bool ref, int step_end, long long budget,
                          long long max_ns) {
    RunState& R = h->run;
    const int ntraj = R.args.num_trajectories;
    for (int g = 0; g < R.ngroups; g++) {
        KernelGroup& G = R.grp[g];
        cudaStream_t s = g == 0 ? h->st : h->st2;
        if (g == 1) {
            cudaEventRecord(h->fork, h->st);
            cudaStreamWaitEvent(h->st2, h->fork, 0);
        }
        // a group without a device list runs trajectories 0 .. ntraj-1
        const int n = G.d_list ? (int)G.list.size() : ntraj;
        const int* tl = G.d_list;
        if (G.batch && G.warps > 1)
            launch_nsm_batchw(ref, G.variant, G.warps, G.warp_smem, h->d_trajs, h->d_insts, n,
                              step_end, h->dt, budget, max_ns, h->d_work + g, h->num_sms, tl, s);
        else if (G.batch)
            launch_nsm_batch(ref, G.variant, G.warp_smem, h->d_trajs, h->d_insts, n, step_end,
                             h->dt, budget, max_ns, h->d_work + g, h->num_sms, tl, s);
        else
            launch_nsm_advance(ref, G.smem_state, G.variant, G.warp_smem, G.wpb, h->d_trajs,
                               h->d_insts, n, step_end, h->dt, budget, max_ns, h->d_work + g,
                               h->num_sms, tl, s);
    }
    if (R.ngroups == 2) {
        cudaEventRecord(h->join, h->st2);
        cudaStreamWaitEvent(h->st, h->join, 0);
    }
}

int sp_run_start(sp_handle* h, const sp_run_args* a, sp_outputs* out) {
    if (!h) return SP_E_INVALID;
    if (!a || a->num_trajectories < 1 || !a->seeds || !a->u0)
        return fail(h, SP_E_INVALID, "sp_run: num_trajectories, seeds and u0 are required");
    if (a->selection != SP_SELECT_EXACT && a->selection != SP_SELECT_REFERENCE)
        return fail(h, SP_E_INVALID, "sp_run: unknown selection mode");
    SP_CUDA_TRY(cudaSetDevice(h->device));
    if (h->run.active) run_release(h);
    RunState& R = h->run;
    R = RunState{};
    R.wall0 = std::chrono::steady_clock::now();
    R.args = *a;
    R.out = out ? *out : sp_outputs{};
    const int ntraj = a->num_trajectories;
    const int ninst = (int)h->inst.size();
    R.inst.assign(ntraj, 0);
    for (int j = 0; j < ntraj; j++) {
        R.inst[j] = a->instance ? a->instance[j] : 0;
        if (R.inst[j] < 0 || R.inst[j] >= ninst) return fail(h, SP_E_INVALID, "instance index out of range");
        if (h->inst[R.inst[j]].S == 0) return fail(h, SP_E_INVALID, "sp_run: model has no species");
        if (!h->inst[R.inst[j]].is_static) R.coupled = true;
    }
    if (R.coupled) {
        // one shared flow: every trajectory runs the same moving instance
        for (int j = 1; j < ntraj; j++)
            if (R.inst[j] != R.inst[0])
                return fail(h, SP_E_INVALID,
                            "sp_run: the trajectories of a moving-domain model must all run one instance");
        R.cinst = R.inst[0];
        int rc0 = sdpd_reset(h->inst[R.cinst].sdpd, &h->err);
        if (rc0) return rc0;
    }
    int rc = ensure_traj(h, ntraj, R.inst.data());
    if (rc) return rc;
    for (int j = 0; j < ntraj; j++) {
        NsmTraj& T = h->h_trajs[j];
        T.key0 = (uint32_t)a->seeds[j];
        T.key1 = (uint32_t)(a->seeds[j] >> 32);
        T.status = SP_TRAJ_OK;
        T.step = 0;
        T.err_voxel = -1;
        T.evn = 0;
        T.nrx = T.ndf = 0;
        T.t_last = 0.0;
        T.a_tot = 0.0;
        T.bscale = 20.0f;
        T.nbatch = T.ncand = 0;
    }
    cudaStream_t st = h->st;
    R.active = true;
    h->launches = 0;
    h->adv_ms = 0;
    SP_CUDA_TRY(cudaEventRecord(h->e0, st));
    SP_CUDA_TRY(cudaMemcpyAsync(h->d_trajs, h->h_trajs.data(), sizeof(NsmTraj) * ntraj,
                                cudaMemcpyHostToDevice, st));
    auto dmalloc = [&](void** p, size_t bytes) -> int {
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) { run_release(h); return spg_set_cuda_error(h, e, "cudaMalloc", __FILE__, __LINE__); }
        R.tmp.push_back(*p);
        return SP_OK;
    };
    // initial counts (u0 per instance)
    std::vector<const uint32_t*> u0ptr(ninst, nullptr);
    for (int i = 0; i < ninst; i++) {
        const Instance& I = h->inst[i];
        if (!a->u0[i]) continue;
        if (a->buffers_on_device) {
            u0ptr[i] = a->u0[i];
        } else {
            void* d = nullptr;
            if ((rc = dmalloc(&d, sizeof(uint32_t) * (size_t)I.N * I.S))) return rc;
            cudaMemcpyAsync(d, a->u0[i], sizeof(uint32_t) * (size_t)I.N * I.S, cudaMemcpyHostToDevice, st);
            u0ptr[i] = (const uint32_t*)d;
        }
    }
    for (int j = 0; j < ntraj; j++)
        if (!u0ptr[R.inst[j]]) { run_release(h); return fail(h, SP_E_INVALID, "u0 missing for an instance in use"); }
    // deterministic chemistry: C = u0, Q = 0 for every instance in use with enable_pde
    {
        std::vector<char> used(ninst, 0);
        for (int j = 0; j < ntraj; j++) used[R.inst[j]] = 1;
        for (int i = 0; i < ninst; i++) {
            Instance& I = h->inst[i];
            if (!used[i] || !I.pde) continue;
            R.chem = true;
            std::vector<double> c0((size_t)I.N * I.S);
            std::vector<uint32_t> u(c0.size());
            cudaError_t e = cudaSuccess;
            if (a->buffers_on_device)
                e = cudaMemcpy(u.data(), u0ptr[i], sizeof(uint32_t) * u.size(), cudaMemcpyDeviceToHost);
            else
                std::memcpy(u.data(), a->u0[i], sizeof(uint32_t) * u.size());
            for (size_t q = 0; q < c0.size(); q++) c0[q] = (double)u[q];   // C = u0 (template :77-80)
            if (e == cudaSuccess)
                e = cudaMemcpy(I.chem.C, c0.data(), sizeof(double) * c0.size(), cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = cudaMemsetAsync(I.chem.Q, 0, sizeof(double) * c0.size(), st);
            if (e != cudaSuccess) {
                run_release(h);
                return spg_set_cuda_error(h, e, "chemistry reset", __FILE__, __LINE__);
            }
        }
    }
    R.chem_step = 0;
    const uint32_t** d_u0 = nullptr;
    if ((rc = dmalloc((void**)&d_u0, sizeof(void*) * ninst))) return rc;
    cudaMemcpyAsync(d_u0, u0ptr.data(), sizeof(void*) * ninst, cudaMemcpyHostToDevice, st);
    int max_leaf = 0, max_levels = 0;
    for (int j = 0; j < ntraj; j++) {
        const NsmInstance& d = h->inst[R.inst[j]].desc;
        max_leaf = std::max(max_leaf, d.leaf_stride);
        max_levels = std::max(max_levels, d.levels);
    }
    // kernel groups: with the default policy, domains of >= 2,048 voxels
    // (64 voxel groups) run the speculative batch kernel and smaller ones a
    // sequential kernel, the two groups concurrently on two streams
    std::vector<int> all(ntraj), big, small;
    for (int j = 0; j < ntraj; j++) all[j] = j;
    if (h->opt.nsm_variant == 0) {
        for (int j = 0; j < ntraj; j++) {
            const Instance& I = h->inst[R.inst[j]];
            const bool eligible = I.N >= 2048 && net_variant(h, {j}, R.inst) != 0 &&
                                  nsm_batch_smem(I.desc) <= 200 * 1024;
            (eligible ? big : small).push_back(j);
        }
    }
    if (!big.empty() && !small.empty()) {
        R.ngroups = 2;
        rc = choose_group(h, R, big, true, R.grp[0]);
        if (rc == SP_OK) rc = choose_group(h, R, small, false, R.grp[1]);
    } else {
        R.ngroups = 1;
        const bool want_batch = h->opt.nsm_variant == 2 || h->opt.nsm_variant >= 4 ||
                                (h->opt.nsm_variant == 0 && !big.empty());
        rc = choose_group(h, R, all, want_batch, R.grp[0]);
    }
    if (rc) { run_release(h); return rc; }
    // the tuner needs a few intervals to spare: one batch group, static
    // domains, default policy, at least six output intervals
    R.tune = WarpTuner{};
    if (h->opt.nsm_variant == 0 && R.ngroups == 1 && R.grp[0].batch && !R.coupled &&
        (int)h->output_steps.size() >= 7) {
        R.tune.on = true;
        set_warps(h, R, R.grp[0], WarpTuner::widths[0]);
    }
    h->last_kernel = kernel_kind(R);
    R.max_leaf = max_leaf;
    R.max_levels = max_levels;
    R.rebuild_variant = R.coupled ? net_variant(h, all, R.inst) : 0;
    launch_nsm_init(h->d_trajs, h->d_insts, ntraj, max_leaf, max_levels, d_u0, !R.coupled, st);
    h->launches += R.coupled ? 1 : 3;
    if (R.ngroups == 2) {
        // largest total propensity first, so the longest trajectories start
        // first (longest-processing-time order)
        SP_CUDA_TRY(cudaMemcpyAsync(h->h_trajs.data(), h->d_trajs, sizeof(NsmTraj) * ntraj,
                                    cudaMemcpyDeviceToHost, st));
        SP_CUDA_TRY(cudaStreamSynchronize(st));
        for (int g = 0; g < 2; g++) {
            KernelGroup& G = R.grp[g];
            std::stable_sort(G.list.begin(), G.list.end(), [&](int a, int b) {
                return h->h_trajs[a].a_tot > h->h_trajs[b].a_tot;
            });
        }
        // Skewed ensembles: when the largest initial total propensity is at
        // least 8 times the 90th percentile, the run takes as long as its
        // heaviest dependent chains.  Every trajectory then runs on the 2-warp
        // batch kernel in one group, heaviest first, so that no concurrent
        // kernel group shares the SMs of those chains.  Measured on the
        // 4,096-instance uneven ensemble, one interval of 0.01: every
        // trajectory on 2 warps 9.0 s, on 4 warps 10.4 s, on 1 warp 11.7 s;
        // the heaviest on 4 warps beside a 1-warp group 11.2 s.  Those chains
        // are sparse: a batch accepts about 11 events whatever its width, and
        // a 2-warp batch costs less.
        if (h->opt.nsm_variant == 0) {
            std::vector<double> at(ntraj);
            for (int j = 0; j < ntraj; j++) at[j] = h->h_trajs[j].a_tot;
            std::vector<double> srt = at;
            const size_t k90 = (size_t)(0.9 * (double)(ntraj - 1));
            std::nth_element(srt.begin(), srt.begin() + k90, srt.end());
            const double p90 = srt[k90];
            const double amax = *std::max_element(at.begin(), at.end());
            if (amax > 0.0 && amax >= 8.0 * p90) {
                // (kept as two groups when one batch group cannot hold every
                // domain's queue in shared memory)
                KernelGroup one;
                const std::string err0 = h->err;
                if (choose_group(h, R, all, true, one) == SP_OK && one.batch) {
                    set_warps(h, R, one, 2);
                    std::stable_sort(one.list.begin(), one.list.end(),
                                     [&](int a, int b) { return at[a] > at[b]; });
                    R.grp[0] = one;
                    R.grp[1] = KernelGroup{};
                    R.ngroups = 1;
                }
                h->err = err0;
            }
        }
        h->last_kernel = kernel_kind(R);
        for (int g = 0; g < R.ngroups; g++) {
            KernelGroup& G = R.grp[g];
            if ((rc = dmalloc((void**)&G.d_list, sizeof(int) * G.list.size()))) return rc;
            SP_CUDA_TRY(cudaMemcpyAsync(G.d_list, G.list.data(), sizeof(int) * G.list.size(),
                                        cudaMemcpyHostToDevice, st));
        }
    }
    // output buffers
    const int nout = (int)h->output_steps.size();
    std::vector<long long> count_off(ntraj), mom_off(ninst);
    R.ctot = 0;
    R.mtot = 0;
    for (int j = 0; j < ntraj; j++) {
        count_off[j] = R.ctot;
        R.ctot += (long long)nout * h->inst[R.inst[j]].N * h->inst[R.inst[j]].S;
    }
    for (int i = 0; i < ninst; i++) {
        mom_off[i] = R.mtot;
        R.mtot += (long long)nout * h->inst[i].N * h->inst[i].S;
    }
    R.want_counts = a->want_counts && out && out->counts;
    R.want_mom = a->want_moments && out && out->moments;
    if (R.want_counts) {
        if (a->buffers_on_device) R.d_counts = out->counts;
        else if ((rc = dmalloc((void**)&R.d_counts, sizeof(int32_t) * R.ctot))) return rc;
        if ((rc = dmalloc((void**)&R.d_coff, sizeof(long long) * ntraj))) return rc;
        cudaMemcpyAsync(R.d_coff, count_off.data(), sizeof(long long) * ntraj, cudaMemcpyHostToDevice, st);
    }
    if (R.want_mom) {
        if (a->buffers_on_device) R.d_mom = (long long*)out->moments;
        else if ((rc = dmalloc((void**)&R.d_mom, sizeof(long long) * 2 * R.mtot))) return rc;
        if ((rc = dmalloc((void**)&R.d_moff, sizeof(long long) * ninst))) return rc;
        cudaMemcpyAsync(R.d_moff, mom_off.data(), sizeof(long long) * ninst, cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(R.d_mom, 0, sizeof(long long) * 2 * R.mtot, st);
    }
    R.want_part = R.coupled && a->want_particles && out &&
                  (out->particle_x || out->particle_v || out->particle_rho);
    if (R.want_part) {
        // particle outputs: [sum_i num_outputs * N_i (* 3)], instance-major
        R.ptot = 0;
        for (int i = 0; i < ninst; i++) {
            if (i == R.cinst) R.poff = R.ptot;
            R.ptot += (long long)nout * h->inst[i].N;
        }
        if (a->buffers_on_device) {
            R.d_px = out->particle_x;
            R.d_pv = out->particle_v;
            R.d_prho = out->particle_rho;
        } else {
            if (out->particle_x && (rc = dmalloc((void**)&R.d_px, sizeof(double) * 3 * R.ptot))) return rc;
            if (out->particle_v && (rc = dmalloc((void**)&R.d_pv, sizeof(double) * 3 * R.ptot))) return rc;
            if (out->particle_rho && (rc = dmalloc((void**)&R.d_prho, sizeof(double) * R.ptot))) return rc;
        }
    }
    R.want_chem = R.chem && a->want_chem && out && out->chem;
    if (R.want_chem) {
        R.chem_off.assign(ninst, 0);
        R.chem_tot = 0;
        for (int i = 0; i < ninst; i++) {
            R.chem_off[i] = R.chem_tot;
            R.chem_tot += (long long)nout * h->inst[i].N * h->inst[i].S;
        }
        if (a->buffers_on_device) R.d_chem = out->chem;
        else if ((rc = dmalloc((void**)&R.d_chem, sizeof(double) * R.chem_tot))) return rc;
        cudaMemsetAsync(R.d_chem, 0, sizeof(double) * R.chem_tot, st);
    }
    R.step = 0;
    R.next_out = 0;
    R.result = SP_OK;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { run_release(h); return spg_set_cuda_error(h, e, "sp_run_start", __FILE__, __LINE__); }
    // outputs at step 0 need no events
    return sp_run_continue(h, 0);
}

// Deterministic chemistry of the static-domain instances of the run, steps
// R.chem_step .. target-1: per step the half step from the previous step's
// fluxes with the boundary conditions (take_step1, simulate.cpp:81-88), the
// fluxes from the fixed neighbour lists (model.cpp:151-189, at t = step*dt),
// and the second half step (take_step2, simulate.cpp:166-171).
static void chem_steps_static(sp_handle* h, int target) {
    RunState& R = h->run;
    if (!R.chem || R.coupled) return;
    std::vector<char> used(h->inst.size(), 0);
    for (int j : R.inst) used[j] = 1;
    for (size_t i = 0; i < h->inst.size(); i++) {
        Instance& I = h->inst[i];
        if (!used[i] || !I.pde || !I.is_static) continue;
        for (int step = R.chem_step; step < target; step++) {
            chem_launch_half(I.chem, I.x, step == 0, true, h->st);
            chem_launch_flux_d(I.chem, I.nbr_cnt, I.nbr_idx, I.nbr_dist, I.nbr_dwdr, I.K, I.mass,
                               I.rho, h->dt * (double)step, h->st);
            chem_launch_half(I.chem, I.x, false, false, h->st);
            h->launches += 3;
        }
    }
    if (target > R.chem_step) R.chem_step = target;
}

// the concentrations of every instance with chemistry into output k
static void chem_snapshot(sp_handle* h, int k) {
    RunState& R = h->run;
    if (!R.want_chem) return;
    std::vector<char> used(h->inst.size(), 0);
    for (int j : R.inst) used[j] = 1;
    for (size_t i = 0; i < h->inst.size(); i++) {
        const Instance& I = h->inst[i];
        if (!used[i] || !I.pde) continue;
        const size_t n = (size_t)I.N * I.S;
        cudaMemcpyAsync(R.d_chem + R.chem_off[i] + (size_t)k * n, I.chem.C, sizeof(double) * n,
                        cudaMemcpyDeviceToDevice, h->st);
    }
}

// one flow step with the chemistry interleaved as the reference's substeps
static void flow_chem_step(sp_handle* h, Instance& I) {
    const SdpdLists L = sdpd_lists(I.sdpd);
    const int step = L.step;
    sdpd_enqueue_phase(I.sdpd, 0);
    if (L.f64) chem_launch_half4d(I.chem, (const double*)L.pos, step == 0, true, h->st);
    else chem_launch_half4f(I.chem, (const float*)L.pos, step == 0, true, h->st);
    sdpd_enqueue_phase(I.sdpd, 1);
    if (L.f64)
        chem_launch_flux_d(I.chem, L.count, L.idx, (const double*)L.dist, (const double*)L.dwdr,
                           L.kcap, (const double*)L.mass, (const double*)L.rho,
                           h->dt * (double)step, h->st);
    else
        chem_launch_flux_f(I.chem, L.count, L.idx, (const float*)L.dist, (const float*)L.dwdr,
                           L.kcap, (const float*)L.mass, (const float*)L.rho,
                           h->dt * (double)step, h->st);
    sdpd_enqueue_phase(I.sdpd, 2);
    if (L.f64) chem_launch_half4d(I.chem, (const double*)L.pos, false, false, h->st);
    else chem_launch_half4f(I.chem, (const float*)L.pos, false, false, h->st);
}

// Moving domain with species, steps R.step .. target-1 (simulate_threads.cpp:
// 232-281 with simulate_rdme.cpp:53-68 on a non-static domain): per step the
// SDPD step, the diffusion tables from its force-pass lists, the volumes from
// the end-of-step density, every trajectory's queue rebuilt at step*dt
// (Philox build index = step) and its events up to (step+1)*dt.  Statuses and
// the flow's error flags are read once, at the target output.
static int coupled_steps(sp_handle* h, int target, bool ref, long long budget, long long max_ns) {
    RunState& R = h->run;
    Instance& I = h->inst[R.cinst];
    cudaStream_t st = h->st;
    const int ntraj = R.args.num_trajectories;
    cudaEventRecord(h->ea, st);
    while (R.step < target) {
        if (I.pde) flow_chem_step(h, I);
        else sdpd_enqueue_step(I.sdpd);
        const SdpdLists L = sdpd_lists(I.sdpd);
        if (L.f64)
            launch_diffusion_tables(I.N, I.S, I.T, I.K, I.type, L.count, L.idx,
                                    (const double*)L.dij, I.diffusion, I.ddiag, I.cdf, I.cdfj, st);
        else
            launch_diffusion_tables_f32(I.N, I.S, I.T, I.K, I.type, L.count, L.idx,
                                        (const float*)L.dij, I.diffusion, I.ddiag, I.cdf, I.cdfj,
                                        st);
        sdpd_launch_volumes(I.sdpd, I.mass, I.vol, I.ivol);
        launch_nsm_rebuild(h->d_trajs, h->d_insts, ntraj, R.max_leaf, R.max_levels,
                           h->dt * (double)R.step, (uint32_t)R.step, R.rebuild_variant, st);
        launch_groups(h, ref, R.step + 1, budget, max_ns);
        h->launches += kSdpdLaunchesPerStep + 1 + 1 + 3 + 1;
        R.step++;
    }
    cudaEventRecord(h->eb, st);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { run_release(h); return spg_set_cuda_error(h, e, "coupled step", __FILE__, __LINE__); }
    int rc = sdpd_check_flag(I.sdpd, &h->err);   // synchronises the stream
    if (rc == SP_E_CUDA) { run_release(h); return rc; }
    if (rc != SP_OK) { R.result = rc; return SP_OK; }
    e = cudaMemcpyAsync(h->h_trajs.data(), h->d_trajs, sizeof(NsmTraj) * ntraj,
                        cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { run_release(h); return spg_set_cuda_error(h, e, "coupled step sync", __FILE__, __LINE__); }
    float ms = 0;
    cudaEventElapsedTime(&ms, h->ea, h->eb);
    h->adv_ms += ms;
    // a step's events run in one launch: an exhausted budget or deadline
    // there is an error, not a pause
    for (int j = 0; j < ntraj; j++)
        if (h->h_trajs[j].status != SP_TRAJ_OK) R.result = SP_E_TRAJECTORY;
    if (R.result == SP_OK && R.args.timeout_s > 0) {
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - R.wall0).count();
        if (el > R.args.timeout_s) R.result = SP_E_TIMEOUT;
    }
    return SP_OK;
}

int sp_run_continue(sp_handle* h, int32_t num_outputs) {
    if (!h) return SP_E_INVALID;
    RunState& R = h->run;
    if (!R.active) return fail(h, SP_E_INVALID, "sp_run_continue: no run in progress");
    if (num_outputs < 0) return fail(h, SP_E_INVALID, "sp_run_continue: negative output count");
    SP_CUDA_TRY(cudaSetDevice(h->device));
    cudaStream_t st = h->st;
    const int ntraj = R.args.num_trajectories;
    const int nout = (int)h->output_steps.size();
    const bool ref = R.args.selection == SP_SELECT_REFERENCE;
    const long long budget = h->opt.event_budget > 0 ? h->opt.event_budget : (1ll << 62);
    const long long max_ns = 2000000000ll;
    int done = 0;
    h->launches = 0;
    h->adv_ms = 0;
    SP_CUDA_TRY(cudaEventRecord(h->e0, st));
    while (R.next_out < nout && R.result == SP_OK) {
        const int target = h->output_steps[R.next_out];
        if (target > 0 && R.coupled) {
            if (done >= num_outputs) break;
            const int rc = coupled_steps(h, target, ref, budget, max_ns);
            if (rc != SP_OK) return rc;
            done++;
        } else if (target > 0) {
            if (done >= num_outputs) break;
            long long ev0 = 0;
            double int_ms = 0;
            if (R.tune.on) {
                set_warps(h, R, R.grp[0], WarpTuner::widths[R.tune.stage]);
                for (int j = 0; j < ntraj; j++) ev0 += h->h_trajs[j].nrx + h->h_trajs[j].ndf;
            }
            for (;;) {
                cudaEventRecord(h->ea, st);
                launch_groups(h, ref, target, budget, max_ns);
                cudaEventRecord(h->eb, st);
                h->launches += R.ngroups;
                cudaError_t e = cudaGetLastError();
                if (e != cudaSuccess) { run_release(h); return spg_set_cuda_error(h, e, "nsm_advance", __FILE__, __LINE__); }
                e = cudaMemcpyAsync(h->h_trajs.data(), h->d_trajs, sizeof(NsmTraj) * ntraj,
                                    cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
                if (e != cudaSuccess) { run_release(h); return spg_set_cuda_error(h, e, "nsm_advance sync", __FILE__, __LINE__); }
                float ms = 0;
                cudaEventElapsedTime(&ms, h->ea, h->eb);
                h->adv_ms += ms;
                int_ms += ms;
                bool again = false;
                for (int j = 0; j < ntraj; j++) {
                    NsmTraj& T = h->h_trajs[j];
                    if (T.status == SP_TRAJ_BUDGET_EXHAUSTED) {
                        T.status = SP_TRAJ_OK;
                        again = true;
                    } else if (T.status != SP_TRAJ_OK) {
                        R.result = SP_E_TRAJECTORY;
                    }
                }
                if (R.result != SP_OK) break;
                if (R.args.timeout_s > 0) {
                    const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - R.wall0).count();
                    if (el > R.args.timeout_s) { R.result = SP_E_TIMEOUT; break; }
                }
                if (!again) break;
                // resume: statuses were reset on the host copy
                cudaMemcpyAsync(h->d_trajs, h->h_trajs.data(), sizeof(NsmTraj) * ntraj,
                                cudaMemcpyHostToDevice, st);
            }
            if (R.tune.on && R.result == SP_OK) {
                long long ev1 = 0;
                for (int j = 0; j < ntraj; j++) ev1 += h->h_trajs[j].nrx + h->h_trajs[j].ndf;
                R.tune.rate[R.tune.stage] = int_ms > 0 ? (double)(ev1 - ev0) / int_ms : 0.0;
                if (++R.tune.stage == 3) {
                    int best = 0;
                    for (int k = 1; k < 3; k++)
                        if (R.tune.rate[k] > R.tune.rate[best]) best = k;
                    set_warps(h, R, R.grp[0], WarpTuner::widths[best]);
                    R.tune.on = false;
                    h->last_kernel = kernel_kind(R);
                }
            }
            done++;
        }
        if (R.result != SP_OK) break;
        chem_steps_static(h, target);
        chem_snapshot(h, R.next_out);
        if (R.want_counts || R.want_mom) {
            launch_nsm_snapshot(h->d_trajs, h->d_insts, ntraj, R.want_counts ? R.d_counts : nullptr,
                                R.d_coff, R.want_mom ? R.d_mom : nullptr, R.d_moff, R.next_out, st);
            h->launches++;
        }
        if (R.want_part) {
            const long long o = R.poff + (long long)R.next_out * h->inst[R.cinst].N;
            sdpd_launch_state_out(h->inst[R.cinst].sdpd, R.d_px ? R.d_px + 3 * o : nullptr,
                                  R.d_pv ? R.d_pv + 3 * o : nullptr,
                                  R.d_prho ? R.d_prho + o : nullptr);
            h->launches++;
        }
        R.next_out++;
    }
    cudaEventRecord(h->e1, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { run_release(h); return spg_set_cuda_error(h, e, "sp_run_continue", __FILE__, __LINE__); }
    float ms = 0;
    cudaEventElapsedTime(&ms, h->e0, h->e1);
    h->last_ms = ms;
    h->last_launches = h->launches;
    if (R.result == SP_E_TRAJECTORY) {
        for (int j = 0; j < ntraj; j++)
            if (h->h_trajs[j].status != SP_TRAJ_OK) {
                char b[256];
                snprintf(b, sizeof b, "trajectory %d stopped with status %d at voxel %d (t=%g)", j,
                         h->h_trajs[j].status, h->h_trajs[j].err_voxel, h->h_trajs[j].t_last);
                h->err = b;
                break;
            }
    } else if (R.result == SP_E_TIMEOUT) {
        h->err = "sp_run: timeout";
    }
    return R.result;
}

int sp_run_finish(sp_handle* h) {
    if (!h) return SP_E_INVALID;
    RunState& R = h->run;
    if (!R.active) return fail(h, SP_E_INVALID, "sp_run_finish: no run in progress");
    SP_CUDA_TRY(cudaSetDevice(h->device));
    cudaStream_t st = h->st;
    const int ntraj = R.args.num_trajectories;
    if (!R.args.buffers_on_device) {
        if (R.want_counts)
            cudaMemcpyAsync(R.out.counts, R.d_counts, sizeof(int32_t) * R.ctot, cudaMemcpyDeviceToHost, st);
        if (R.want_mom)
            cudaMemcpyAsync(R.out.moments, R.d_mom, sizeof(long long) * 2 * R.mtot, cudaMemcpyDeviceToHost, st);
        if (R.want_chem)
            cudaMemcpyAsync(R.out.chem, R.d_chem, sizeof(double) * R.chem_tot,
                            cudaMemcpyDeviceToHost, st);
        if (R.want_part) {
            const long long n = (long long)h->output_steps.size() * h->inst[R.cinst].N;
            if (R.d_px)
                cudaMemcpyAsync(R.out.particle_x + 3 * R.poff, R.d_px + 3 * R.poff,
                                sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st);
            if (R.d_pv)
                cudaMemcpyAsync(R.out.particle_v + 3 * R.poff, R.d_pv + 3 * R.poff,
                                sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st);
            if (R.d_prho)
                cudaMemcpyAsync(R.out.particle_rho + R.poff, R.d_prho + R.poff,
                                sizeof(double) * n, cudaMemcpyDeviceToHost, st);
        }
    }
    cudaMemcpyAsync(h->h_trajs.data(), h->d_trajs, sizeof(NsmTraj) * ntraj, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    const int result = R.result;
    if (R.out.event_counts)
        for (int j = 0; j < ntraj; j++) {
            R.out.event_counts[2 * j] = h->h_trajs[j].nrx;
            R.out.event_counts[2 * j + 1] = h->h_trajs[j].ndf;
        }
    run_release(h);
    if (e != cudaSuccess) return spg_set_cuda_error(h, e, "sp_run_finish", __FILE__, __LINE__);
    return result;
}

int sp_run(sp_handle* h, const sp_run_args* a, sp_outputs* out) {
    int rc = sp_run_start(h, a, out);
    if (rc != SP_OK) {
        if (h && h->run.active) sp_run_finish(h);
        return rc;
    }
    double ms0 = h->last_ms;
    long long l0 = h->last_launches;
    const int rc2 = sp_run_continue(h, 1 << 30);
    const double adv = h->adv_ms;
    h->last_ms += ms0;
    h->last_launches += l0;
    if (!h->run.active) return rc2;   // released on a CUDA error; keep its message
    const int rc3 = sp_run_finish(h);
    h->adv_ms = adv;
    return rc2 != SP_OK ? rc2 : rc3;
}

int sp_last_profile(sp_handle* h, sp_profile* p) {
    if (!h || !p) return SP_E_INVALID;
    p->total_ms = h->last_ms;
    p->kernel_ms = h->adv_ms;
    p->launches = h->last_launches;
    p->kernel = h->last_kernel;
    return SP_OK;
}

int sp_status(sp_handle* h, int32_t traj, sp_traj_status* st) {
    if (!h || !st) return SP_E_INVALID;
    if (traj < 0 || traj >= (int)h->h_trajs.size()) return fail(h, SP_E_INVALID, "trajectory out of range");
    const NsmTraj& T = h->h_trajs[traj];
    st->code = T.status;
    st->voxel = T.err_voxel;
    st->time = T.t_last;
    st->events = T.nrx + T.ndf;
    st->batches = T.nbatch;
    st->candidates = T.ncand;
    return SP_OK;
}

const char* sp_last_error(sp_handle* h) { return h ? h->err.c_str() : "null handle"; }

void sp_destroy(sp_handle* h) {
    if (!h) return;
    if (!h->st) {   // never reached the device (argument errors)
        delete h;
        return;
    }
    cudaSetDevice(h->device);
    if (h->st) cudaStreamSynchronize(h->st);
    if (h->run.active) run_release(h);
    for (Instance& I : h->inst)
        if (I.sdpd) sdpd_destroy(I.sdpd);
    for (void* p : h->allocs) cudaFree(p);
    if (h->traj_mem) cudaFree(h->traj_mem);
    if (h->e0) cudaEventDestroy(h->e0);
    if (h->e1) cudaEventDestroy(h->e1);
    if (h->ea) cudaEventDestroy(h->ea);
    if (h->eb) cudaEventDestroy(h->eb);
    if (h->fork) cudaEventDestroy(h->fork);
    if (h->join) cudaEventDestroy(h->join);
    if (h->st2) cudaStreamDestroy(h->st2);
    if (h->st) cudaStreamDestroy(h->st);
    delete h;
}

int sp_get_neighbors(sp_handle* h, int32_t inst, int32_t kmax, int32_t* count, int32_t* idx,
                     double* dist, double* dWdr, double* Dij) {
    if (!h || inst < 0 || inst >= (int)h->inst.size() || !count || !idx) return SP_E_INVALID;
    Instance& I = h->inst[inst];
    SP_CUDA_TRY(cudaSetDevice(h->device));
    const int N = I.N;
    int K = I.K;
    const int *d_cnt = I.nbr_cnt, *d_idx = I.nbr_idx;
    const double *d_dist = I.nbr_dist, *d_dw = I.nbr_dwdr, *d_dij = I.nbr_dij;
    if (!I.is_static) return sdpd_copy_neighbors(I.sdpd, kmax, count, idx, dist, dWdr, Dij, &h->err);
    std::vector<int> c(N), ix((size_t)N * K);
    std::vector<double> d1((size_t)N * K), d2((size_t)N * K), d3((size_t)N * K);
    SP_CUDA_TRY(cudaMemcpy(c.data(), d_cnt, sizeof(int) * N, cudaMemcpyDeviceToHost));
    SP_CUDA_TRY(cudaMemcpy(ix.data(), d_idx, sizeof(int) * N * (size_t)K, cudaMemcpyDeviceToHost));
    if (d_dist) SP_CUDA_TRY(cudaMemcpy(d1.data(), d_dist, sizeof(double) * N * (size_t)K, cudaMemcpyDeviceToHost));
    if (d_dw) SP_CUDA_TRY(cudaMemcpy(d2.data(), d_dw, sizeof(double) * N * (size_t)K, cudaMemcpyDeviceToHost));
    if (d_dij) SP_CUDA_TRY(cudaMemcpy(d3.data(), d_dij, sizeof(double) * N * (size_t)K, cudaMemcpyDeviceToHost));
    for (int i = 0; i < N; i++) {
        if (c[i] > kmax) return fail(h, SP_E_INVALID, "kmax smaller than a neighbour count");
        count[i] = c[i];
        for (int k = 0; k < c[i]; k++) {
            const size_t s = (size_t)i * K + k, o = (size_t)i * kmax + k;
            idx[o] = ix[s];
            if (dist) dist[o] = d1[s];
            if (dWdr) dWdr[o] = d2[s];
            if (Dij) Dij[o] = d3[s];
        }
    }
    return SP_OK;
}

int sp_get_ddiag(sp_handle* h, int32_t inst, double* ddiag) {
    if (!h || inst < 0 || inst >= (int)h->inst.size() || !ddiag) return SP_E_INVALID;
    Instance& I = h->inst[inst];
    if (!I.ddiag) return fail(h, SP_E_INVALID, "instance has no diffusion tables");
    std::vector<float> f((size_t)I.N * I.S);
    SP_CUDA_TRY(cudaMemcpy(f.data(), I.ddiag, sizeof(float) * f.size(), cudaMemcpyDeviceToHost));
    for (size_t e = 0; e < f.size(); e++) ddiag[e] = f[e];
    return SP_OK;
}

int sp_get_particles(sp_handle* h, int32_t inst, double* x, double* v, double* rho) {
    if (!h || inst < 0 || inst >= (int)h->inst.size()) return SP_E_INVALID;
    Instance& I = h->inst[inst];
    SP_CUDA_TRY(cudaSetDevice(h->device));
    if (I.sdpd) {
        return sdpd_get_state(I.sdpd, x, v, rho, &h->err);
    }
    if (x) SP_CUDA_TRY(cudaMemcpy(x, I.x, sizeof(double) * 3 * I.N, cudaMemcpyDeviceToHost));
    if (v) std::memset(v, 0, sizeof(double) * 3 * I.N);
    if (rho) SP_CUDA_TRY(cudaMemcpy(rho, I.rho, sizeof(double) * I.N, cudaMemcpyDeviceToHost));
    return SP_OK;
}

int sp_sdpd_advance(sp_handle* h, int32_t inst, int32_t nsteps) {
    if (!h || inst < 0 || inst >= (int)h->inst.size() || nsteps < 0) return SP_E_INVALID;
    Instance& I = h->inst[inst];
    if (!I.sdpd) return fail(h, SP_E_INVALID, "instance is a static domain");
    SP_CUDA_TRY(cudaSetDevice(h->device));
    double ms = 0;
    long long launches = 0;
    int rc = sdpd_advance(I.sdpd, nsteps, &ms, &launches, &h->err);
    h->last_ms = ms;
    h->last_launches = launches;
    return rc;
}

int sp_last_timing(sp_handle* h, double* ms, int64_t* launches) {
    if (!h) return SP_E_INVALID;
    if (ms) *ms = h->last_ms;
    if (launches) *launches = h->last_launches;
    return SP_OK;
}

}  // extern "C"
