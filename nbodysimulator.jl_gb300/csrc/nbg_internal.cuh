// nbg_internal.cuh - shared declarations and device helpers of libnbg.
//
// Data layout in device memory (one context = one system or a batch of
// replicas, atoms of replica r at [atom0_r, atom0_r + n_r)):
//   x, v, a_old, a_new : double[3 * cols]  (the reference's 3 x n column-major
//                        state, Nose-Hoover column last for a single system)
//   phi, plo           : float4[n] split positions: phi = (hi.xyz, w),
//                        plo = (lo.xyz, flags) with x = hi + lo to ~2^-48
//                        relative. Under cubic boundaries hi is the wrapped
//                        position rounded to a 2^-k grid (k = 23 - ceil(log2 L))
//                        so that hi_i - hi_j and the +-L image shift are exact
//                        in FP32; w is the charge (pair path) or mass (gravity).
//   cell_count/cell_atoms, nbr/nbr_count, xref : cell and Verlet lists.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/nbg.h"

// NVTX ranges in the domain "nbg" around the library's calls and the host
// side of their phases (list build, forces, integration chunks). Without an
// attached tool (Nsight Systems, Nsight Compute) a push or pop is one test of
// a null callback. Inside a stream capture a range marks the capture, not
// the graph's later replays.
inline nvtxDomainHandle_t nbg_nvtx_domain()
{
    static nvtxDomainHandle_t dom = nvtxDomainCreateA("nbg");
    return dom;
}

struct NbgRange {
    explicit NbgRange(const char* name)
    {
        nvtxEventAttributes_t a = {};
        a.version = NVTX_VERSION;
        a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
        a.messageType = NVTX_MESSAGE_TYPE_ASCII;
        a.message.ascii = name;
        nvtxDomainRangePushEx(nbg_nvtx_domain(), &a);
    }
    ~NbgRange() { nvtxDomainRangePop(nbg_nvtx_domain()); }
    NbgRange(const NbgRange&) = delete;
    NbgRange& operator=(const NbgRange&) = delete;
};
#define NBG_RANGE(name) NbgRange nbg_range_scope_(name)

// device status word bits
#define ST_CELL_OVERFLOW 1u
#define ST_NBR_OVERFLOW 2u
#define ST_NONFINITE 4u
#define ST_RANGE 8u
#define ST_SHORT_OVERFLOW 16u  // learned-model short list
#define ST_TIMEOUT 32u         // a bounded wait in a kernel ran out
#define ST_INDEX 64u           // debug builds: a neighbour or cell index out of range
// bits that end a call with an error (the others regrow capacity)
#define ST_FATAL (ST_NONFINITE | ST_RANGE | ST_TIMEOUT | ST_INDEX)

// atom flags (plo.w bits)
#define AF_LJ 1

// relative margin of the FP32 cutoff classification; pairs whose FP32 r^2 lies
// within it of R^2 are classified again with the reference's FP64 arithmetic.
#define CLASSIFY_MARGIN 1.0e-5

// iteration cap of the reference's minimum-image while loops
#define MINIMAGE_MAX_ITERS 65536

struct RepDev {
    int64_t atom0, n;   // atom range of the replica
    double L, invL;     // cubic box
    double box[6];      // general periodic box (lo,hi per axis)
    float Lh, Ll;       // L split on the hi grid: L = Lh + Ll
    float invLf;
    float qscale, qinv; // 2^k and 2^-k of the hi grid
    float lj_lo, lj_hi; // FP32 r^2 below lo: inside; >= hi: outside; else exact
    float el_lo, el_hi;
    float rl2;          // Verlet-list radius^2 (inflated)
    int nc;             // cells per dimension
    int ns;             // cell stencil half-width: cells >= rl / ns (0: one cell holds the replica)
    int cell0;          // first cell of the replica
    double cell_inv;    // nc / L
    double T0, tparam;  // thermostat target and tau / nu / gamma
    double bc1, bsd;    // BAOAB: exp(-gamma dt) and sqrt(1 - c1^2) sqrt(kb T0) for the current dt
    double sigma;       // Langevin noise amplitude (potential systems)
    double sigma_num;   // sqrt(2 gamma kb T) (water)
    double ndf;         // 3N - Nc
    uint64_t seed;
    // fixed-point box coordinates (list path, cubic): q = x / L * 2^32 mod 2^32,
    // so a 32-bit wrapping difference is the minimum image in box units
    // u = L / 2^32; every FP32 constant below is in those units
    double fx_scale;             // 2^32 / L
    float fx_lj_lo, fx_lj_hi;    // classification bands of r^2 (as lj_lo / lj_hi)
    float fx_el_lo, fx_el_hi;
    // The kernel sums, per pair, (2 s^6 - 1) s^6 / r^2 d for LJ and
    // kq_i q_j (rinv^3 - krf) d for electrostatics (box units, s^2 =
    // sigma^2 / r^2, kq_i = k q_i / (u^2 fscale)) and multiplies the sums by
    // fscale (24 eps / u with LJ, else 1) in FP64: the FP32 constants of the
    // pair loop carry no systematic rounding beyond sigma^2's (kept as a
    // hi + lo pair) and the charges'.
    float fx_sig2_hi, fx_sig2_lo;  // sigma^2 / u^2
    float fx_krf;                  // 2 k_rf u^3
    double fx_fscale;
    double fx_kq;                  // k / (u^2 fscale), host FP64: the kernels' kq_i = q_i fx_kq
    float fx_rl2;                  // list radius^2 (inflated), box units
    float fx_disp2;                // (skin/2)^2 in box units, slightly inside (rebuild trigger)
    // cell grid of the persistent ensemble loop's in-kernel list build, per
    // cell-width choice [0]: cells of >= rl over 3^3 cells, [1]: >= rl/2 over
    // 5^3; nc = 1 (ns = 0): one cell holds the replica
    int ens_nc[2], ens_ns[2];
};

// Everything a kernel needs, passed by value.
// Where the step loop leaves saved frames (device memory): with t the step
// index counted from the run's first step t0 (the context's step counter
// keeps running across runs), the state after step t goes to slot
// t / every - first when t is a multiple of every and the slot is below cap.
// every = 0: nothing is saved.
struct FrameSink {
    double* x;  // [cap][3 cols] positions
    double* v;  // [cap][3 cols] velocities
    int64_t every, first, cap;
    int64_t t0;  // absolute step index of the run's initial state
};

struct Dev {
    int64_t n;          // atoms (all replicas)
    int64_t cols;       // state columns (n, +1 with Nose-Hoover)
    int kind, bc, therm, nrep;
    uint32_t pots;
    // parameters
    float lj_sig2, lj_eps24;
    double lj_sig2_d, lj_eps, lj_R2;
    float el_k, el_krf2;          // k and 2 k_rf (reaction field)
    double el_k_d, el_R, el_R2, el_krf, el_crf;
    double G, mu4pi, kb;
    double rOH, aHOH, kbond, kangle;
    double skin_half2;            // (skin/2)^2
    // per atom
    const double* mass;
    const double* inv_mass;
    const double* rsqrt_mass;     // 1 / sqrt(m)
    const double* charge;
    const double* dipole;
    const int* rep_of;
    const RepDev* reps;
    float4* phi;
    float4* plo;
    // fixed-point positions (x, y, z as 32-bit box fractions, w the charge's
    // FP32 bits) for the list force kernel; null where it is not used
    uint4* pfx;
    int split_on;       // the steps also refresh phi / plo (their per-step readers run)
    // lists
    int* cell_count;
    int* cell_n;
    int* cell_atoms;
    int cell_cap;
    int ncell_total;
    int* nbr;           // entry k of atom i at nbr[k * nbr_kstride + i * nbr_istride]
    int* nbr_count;
    int nbr_cap;
    int64_t nbr_kstride;  // n (column-major, thread per atom) or 1 (row-major, lanes per atom)
    int64_t nbr_istride;  // 1 or nbr_cap
    double* xref;
    double* img;                // list path, cubic: per atom the periodic image index fixed at its replica's last list build
    int* rebuild_flag;          // [2][nrep]: per replica, by the parity of the position time index
    const int* cell_rep;        // replica of each cell
    unsigned long long* build_count;
    unsigned* status;
    int64_t* step_dev;          // step counter read by graph-captured kernels
    FrameSink* sink;            // trajectory frames kept on the device (nbg_run)
    // reductions
    double* red_partial;
    double* red_T;      // per replica temperature of the current velocities
    unsigned* red_counter;
    int red_slices;
    // gravity
    int grav_plain;
};

// learned short-range model (k_learned.cu; oracle/learned.py restates it)
#define ML_RD 0.6f     // descriptor cutoff (nm)
#define ML_R0 0.07f    // first radial centre
#define ML_W ((ML_RD - ML_R0) / 23.0f)
#define ML_RS 0.45f    // start of the short-range switch
#define ML_ALPHA 4.0f  // Coulomb screening of the short-range target (1/nm)
#define ML_RHO0 0.1f   // angular envelope widths
#define ML_RHO1 0.2f
#define ML_RHO2 0.3f
#define ML_RHO3 10.0f
#define ML_NTRAIN (64 * 128 + 128 + 128 * 128 + 128 + 128 + 1)  // trainable parameters per species
#define ML_NPARAM (ML_NTRAIN + 2 * 64 + 2)                      // plus mean/sd of inputs and label

struct MLTrainScratch {
    int* idx = nullptr;
    float *xs = nullptr, *a1 = nullptr, *a2 = nullptr, *g1 = nullptr, *g2 = nullptr, *eo = nullptr;
    float* grad = nullptr;
    float* m1[2] = {nullptr, nullptr};  // Adam moments per species
    float* m2[2] = {nullptr, nullptr};
    double* loss = nullptr;
    int B = 0;  // batch capacity of the scratch
};

struct StateView {
    double* x;
    double* v;
    double* a_old;
    double* a_new;
};

struct nbg_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    nbg_system_desc desc{};
    int nrep = 1;
    std::vector<RepDev> reps_h;
    std::vector<double> mass_h, charge_h, dipole_h;
    int64_t n = 0, cols = 0;
    int path = 0;          // PATH_*
    Dev d{};
    StateView st{};        // resident state
    StateView ev{};        // scratch state for nbg_accel / nbg_energy / nbg_pair_list
    bool state_valid = false;
    bool accel_valid = false;
    // x, v, a_old, a_new of each view are one allocation, in that order
    // (the step loop backs up x, v, a_old with one copy)
    double* bk = nullptr;  // backup [4][3 cols]: x, v, a_old, then the r-RESPA slow acceleration
    // an nbg_advance whose last chunk's status word was not read yet; the
    // next call on the context settles it (re-running the chunk after a list
    // overflow, or returning its error)
    bool pending = false;
    double pend_dt = 0.0;
    int64_t pend_steps = 0, pend_step0 = 0;
    // the status of a chunk reaches the host through a pinned, mapped word:
    // a chunk run as one launch (cluster or ensemble loop, chunk_hw) sets its
    // bits there directly, any other deferred chunk copies the device word
    // there; pend_ev follows the chunk, so settling waits for the chunk
    // alone, not for work queued on the stream after it
    unsigned* hw = nullptr;
    unsigned* hw_d = nullptr;  // its device address
    bool chunk_hw = false;
    cudaEvent_t pend_ev = nullptr;
    int64_t step = 0;      // steps taken on the resident state
    int64_t steps_since_build = 0;
    int64_t list_builds = 0;
    int64_t launches = 0;
    // gravity path: bodies padded to npad (multiple of the 256-body tile)
    int64_t npad = 0;
    int grav_chunks = 1;
    int grav_variant = 1;     // k_gravity form (bodies per thread, packed FP32x2)
    // small systems: velocity Verlet in one persistent cluster launch (k_cluster.cu)
    bool cluster_disabled = false;
    bool cluster_ok = false;
    int cluster_size = 0, cluster_per = 0, cluster_lpa = 0, cluster_cap = 0;
    size_t cluster_bytes = 0;
    double* cluster_x = nullptr;  // FP64 positions of the two step parities [2][3n]
    // the lists a cluster launch leaves for the next ([CTA][per][cap], counts,
    // steps since the build); valid only while nothing else changed the state
    int* cluster_lists = nullptr;
    int* cluster_cnt = nullptr;
    double* cluster_xref = nullptr;  // [3n] positions at the cluster lists' build
    int* cluster_since = nullptr;
    bool cluster_lists_valid = false;
    // nbg_accel's cluster launches keep lists of their own (same shapes),
    // valid for any positions within skin/2 of cla_xref
    int* cla_lists = nullptr;
    int* cla_cnt = nullptr;
    double* cla_xref = nullptr;
    bool cla_valid = false;
    // replica ensembles: one persistent launch per chunk of steps, a CTA per
    // replica (k_ensemble.cu)
    bool ens_ok = false, ens_disabled = false;
    bool ens_tuned_off = false;  // nbg_ensemble_tune chose the step graphs over the loop
    bool ens_lists_valid = false;  // the lists, their reference positions and step counts are the loop's
    int ens_lpa = 4, ens_threads = 768, ens_cells = 0;  // form: lanes per atom, threads, cell width (0 = as planned, 1 = rl, 2 = rl/2)
    size_t ens_smem = 0;
    int* ens_order = nullptr;     // replicas, largest first (CTA b runs replica order[b])
    int* ens_since = nullptr;     // per replica: steps since its list build
    uint4* ens_pref = nullptr;    // per atom: fixed-point position at its replica's last build
    // test of the cluster loop's timeout path: the launch after
    // cluster_test_skip others drops the position copies of this step (-1:
    // its last step; -2: none)
    int cluster_test_drop = -2;
    // debug builds: NBG_TEST_PLANT_INDEX=k writes n + k into the first entry
    // of atom 0's Verlet-list row after the next list build outside a stream
    // capture (one shot), for the tests of the index checks
    int plant_index = 0;
    int cluster_test_skip = 0;
    bool grav_uniform = false;  // every body has mass grav_m0: the reduction applies G m
    float grav_far2 = 256.f;    // a tile pair is far when (F g)^2 >= max|r|^2, F = 16
    double grav_m0 = 0.0;
    int list_lpa = 0;         // lanes per atom of k_force_list (1 = thread per atom)
    // the fixed-point, list-staged force kernel (k_force_fx.cu): its tensor
    // map of the list, grid and shared memory for the current form
    alignas(64) unsigned char fx_map[128];
    bool fx_ready = false;     // it runs (else the split-form kernels do)
    bool fx_disabled = false;  // NBG_NO_FX: the split-form kernels only
    bool fx_block_only = false;  // NBG_FX_BLOCK: the per-block staging form for every width
    int fx_grid = 0, fx_nbox = 0;
    size_t fx_smem = 0;
    double* grav_part = nullptr;
    // compensated gravity: bodies re-sorted along a Morton curve every 8th
    // evaluation; far tile pairs take the plain FP32 difference
    bool grav_sort = false;
    unsigned* grav_extent = nullptr;  // half-width of the Morton cube (FP32 bits), found on the device
    unsigned long long* grav_keys[2] = {nullptr, nullptr};
    int* grav_vals[2] = {nullptr, nullptr};  // [1] = the permutation (slot -> body)
    void* grav_sort_tmp = nullptr;
    size_t grav_sort_bytes = 0;
    float4* grav_box = nullptr;       // 2 per 128-body tile
    int64_t grav_evals = 0;           // gravity evaluations issued (the sort runs on every 8th)
    bool grav_perm_valid = false;     // the permutation belongs to the positions being evaluated
    // profiling of the dominant force kernel
    bool profiling = false;
    // captured step graphs (velocity Verlet / Euler-Maruyama)
    cudaGraphExec_t graph = nullptr;
    // nbg_accel on the list path: the whole right-hand side as one graph on
    // pinned staging buffers; the lists are rebuilt only when an atom moved
    // more than skin/2 since they were built for an earlier call's positions
    cudaGraphExec_t accel_graph = nullptr;
    double* hst = nullptr;         // pinned, mapped [3][3 cols] u, v, dv, then the status word (the GPU reads and writes it)
    int64_t* accel_step = nullptr; // device counter of the calls (parity of the rebuild flags)
    bool accel_lists_valid = false;
    int64_t accel_graph_launches = 0;  // kernels per replay
    int64_t graph_steps = 0;     // steps per replay
    int64_t graph_launches = 0;  // kernels per replay
    double graph_dt = 0.0;
    bool graph_sink = false;     // the captured steps save frames
    bool use_graphs = true;
    // trajectory frames on the device: the steps save them while sink_on
    bool sink_on = false;
    double* frames = nullptr;    // [2][frames_cap][3 cols]: positions, then velocities
    int64_t frames_cap = 0;
    bool baoab = false;          // Langevin by BAOAB instead of Euler-Maruyama
    double baoab_dt = -1.0;      // dt of the BAOAB coefficients in the replica table
    // temperature folded into the kick (single system, Berendsen / Nose-Hoover)
    double* kick_part = nullptr;
    unsigned* kick_counter = nullptr;
    int kick_blocks = 0;
    bool T_valid = false;        // red_T holds T of the resident velocities
    int sms = 0;                 // multiprocessors of the device
    // constants of the list-based energy: LJ pairs, and sum of q_i q_j over
    // all non-excluded pairs (i < j)
    int64_t lj_pairs = 0;
    double el_pair_qq = 0.0;
    // learned short-range model (water)
    bool ml_on = false;
    bool ml_attr = false;        // large shared-memory opt-ins done
    float* ml_theta[2] = {nullptr, nullptr};
    __nv_bfloat16* ml_w1[2] = {nullptr, nullptr};
    __nv_bfloat16* ml_w2[2] = {nullptr, nullptr};
    int* ml_snbr = nullptr;
    int* ml_scnt = nullptr;
    int ml_scap = 0;
    float *ml_x = nullptr, *ml_mom = nullptr, *ml_dx = nullptr, *ml_e = nullptr;
    unsigned long long* ml_fq = nullptr;
    float *ml_fsr = nullptr, *ml_esr = nullptr;
    float* ml_X[2] = {nullptr, nullptr};
    float* ml_Y[2] = {nullptr, nullptr};
    int64_t ml_rows[2] = {0, 0}, ml_cap[2] = {0, 0};
    MLTrainScratch ml_ts;
    int64_t ml_adam_t[2] = {0, 0};
    double* ml_judge = nullptr;  // per outer step: sum |F_ml - F_sr|^2, sum |F_sr|^2
    int ml_judge_cap = 0;
    double* ml_a_slow = nullptr;  // r-RESPA slow acceleration (exact non-bonded - learned)
    bool respa_valid = false;     // a_old holds the fast and ml_a_slow the slow acceleration of st
    int respa_mode = 0;           // fast force of respa_valid: 0 learned, 1 exact short-range, 2 none
    std::vector<cudaEvent_t> prof_events;  // start/stop pairs not yet read
    double prof_ms = 0.0;
    int64_t prof_count = 0;
    std::string err;
    std::vector<void*> allocs;
};

enum { PATH_GRAVITY = 0, PATH_LIST = 1, PATH_ALLPAIRS = 2 };

// ---------------------------------------------------------------------
// host-side launchers (one translation unit each)
// ---------------------------------------------------------------------
// Step index of a launch: off + *base (base = the device step counter in a
// captured graph, NULL for a direct launch where off is the absolute step).
struct StepRef {
    int64_t off;
    const int64_t* base;
};

int launch_pack(nbg_ctx* c, const StateView& s);
int launch_gravity(nbg_ctx* c, const StateView& s);
bool cluster_plan(nbg_ctx* c);
// step0: the time index of the state at the launch (for the frame sink)
// (status: the word the launch sets its bits in; the cluster loop also
// writes x, v, a_old of its atoms to the backup before its first step)
int launch_cluster_vv(nbg_ctx* c, const StateView& s, double dt, int64_t nsteps, int rebuild_every, int64_t step0,
                      unsigned* status);
// replica ensembles on the persistent per-replica loop (k_ensemble.cu)
bool ensemble_plan(nbg_ctx* c);
int launch_ensemble(nbg_ctx* c, const StateView& s, double dt, int64_t nsteps, int64_t step0, unsigned* status);
int launch_cluster_accel(nbg_ctx* c, const double* u, double* dv, unsigned* status);
int cluster_launch_floor(nbg_ctx* c, double* us_single, double* us_per_launch);
int launch_allpairs(nbg_ctx* c, const StateView& s);
int launch_list_build(nbg_ctx* c, const StateView& s, bool force, StepRef pos);
#ifdef NBG_DEBUG
int launch_plant_index(nbg_ctx* c, int k);
#endif
int launch_force_list(nbg_ctx* c, const StateView& s);
int fx_prepare(nbg_ctx* c);
int launch_force_fx(nbg_ctx* c, const StateView& s);
int launch_bonded(nbg_ctx* c, const StateView& s);
int launch_drift(nbg_ctx* c, const StateView& s, double dt, StepRef pos);
int launch_temperature(nbg_ctx* c, const double* v);
int launch_kick(nbg_ctx* c, const StateView& s, double dt, bool do_T, bool thermo = true);
int launch_andersen(nbg_ctx* c, const StateView& s, double dt, StepRef step);
int launch_em(nbg_ctx* c, const StateView& s, double dt, StepRef step);
int launch_step_advance(nbg_ctx* c, int64_t by);
int launch_pack_disp(nbg_ctx* c, const double* X, StepRef pos);
int launch_accel_import(nbg_ctx* c, const StateView& s, const double* hu, const double* hv, bool v_read, StepRef pos);
int launch_accel_export(nbg_ctx* c, const StateView& s, double* hdv, double* hv, unsigned* hstat, int64_t* counter);
int launch_counter_advance(nbg_ctx* c, int64_t* counter, int64_t by);
int launch_baoab_drift(nbg_ctx* c, const StateView& s, double dt, StepRef step);
int launch_baoab_kick(nbg_ctx* c, const StateView& s, double dt);
int launch_baoab_kick_drift(nbg_ctx* c, const StateView& s, double dt, StepRef step);
int launch_set_step(nbg_ctx* c, int64_t value);
int launch_save_frame(nbg_ctx* c, const StateView& s, StepRef sr);
int launch_rhs_thermostat(nbg_ctx* c, const StateView& s);
int gravity_plan_chunks(nbg_ctx* c, int64_t npad);
size_t gravity_sort_bytes(int64_t n);
int launch_energy(nbg_ctx* c, const StateView& s, double* out_host /*[8]*/);
int launch_pairs(nbg_ctx* c, const StateView& s, int which, int* out_j, int* out_cnt, int64_t cap_per_atom);

// learned short-range model and r-RESPA (k_learned.cu)
int ml_init_constants();
size_t ml_mlp_smem();
int launch_mlp_attrs(nbg_ctx* c);
int launch_short_list(nbg_ctx* c, StepRef pos, bool force);
int launch_descriptor(nbg_ctx* c, bool raw);
int launch_mlp(nbg_ctx* c);
int launch_ml_force(nbg_ctx* c);
int launch_sr_exact(nbg_ctx* c, float* e_out, float* f_out, double* a_out = nullptr);
int launch_ml_accel(nbg_ctx* c, int mode, double* a);
int launch_ml_force_out(nbg_ctx* c, double* f);
int launch_sr_inner(nbg_ctx* c, StepRef pos, bool force_short, double* a_out);
int launch_sr_accel(nbg_ctx* c, int mode, double* a);
int launch_ml_judge(nbg_ctx* c, StepRef sr, int inner, int slots);
int launch_respa_kick(nbg_ctx* c, double* v, const double* a, double h);
int launch_ml_pack(nbg_ctx* c, int sp);
int launch_ml_collect(nbg_ctx* c, int sp, int64_t off);
int launch_ml_stats(nbg_ctx* c, int sp);
int launch_ml_train_step(nbg_ctx* c, int sp, int B, uint64_t seed, uint64_t batch, float lr, int64_t t_adam);
int launch_ml_batch_grad(nbg_ctx* c, const float* theta, const float* X, const float* Y, int B);

// events around the dominant force kernel when profiling is on
void prof_begin(nbg_ctx* c);
void prof_end(nbg_ctx* c);

// record a CUDA error on the context; returns NBG_ERR_CUDA
int cuda_fail(nbg_ctx* c, cudaError_t e, const char* what);

#define NBG_LAUNCH_CHECK(c, what)                                  \
    do {                                                           \
        (c)->launches++;                                           \
        cudaError_t _e = cudaGetLastError();                       \
        if (_e != cudaSuccess) return cuda_fail((c), _e, (what));  \
    } while (0)

static inline int grid_for(int64_t work, int block)
{
    int64_t g = (work + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 1048576) g = 1048576;
    return (int)g;
}

// ---------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------
#ifdef __CUDACC__

__device__ __forceinline__ int64_t step_of(StepRef r) { return r.off + (r.base ? *r.base : 0); }

__device__ __forceinline__ void status_set(unsigned* st, unsigned bit) { atomicOr(st, bit); }

// Debug builds (nvcc -DNBG_DEBUG, libnbg_debug.so): every neighbour or cell
// index that a kernel reads from a device table is checked against [0, n)
// before it is used; one outside sets ST_INDEX (NBG_ERR_INDEX on the host)
// and is replaced by `safe`, an index known to be valid, so the kernel ends
// without touching memory outside its buffers. Release builds return j.
__device__ __forceinline__ int dbg_index(int j, int64_t n, int safe, unsigned* st)
{
#ifdef NBG_DEBUG
    if (j < 0 || (int64_t)j >= n) {
        status_set(st, ST_INDEX);
        return safe;
    }
#else
    (void)n, (void)safe, (void)st;
#endif
    return j;
}

// x is neither infinite nor NaN (the exponent field is not all ones), by
// integer operations: FP64 compares issue slowly on this GPU
__device__ __forceinline__ bool finite64(double x)
{
    return (__double_as_longlong(x) & 0x7ff0000000000000ll) != 0x7ff0000000000000ll;
}

// The reference's get_interparticle_distance in FP64, no contraction
// (boundary_conditions.jl:111-172). Returns false when a while loop exceeded
// MINIMAGE_MAX_ITERS (non-finite or absurdly distant coordinates).
struct Dist64 {
    double x, y, z, r2;
};

__device__ __forceinline__ bool wrap_cubic64(double& x, double size, double radius)
{
    int it = 0;
    while (x >= radius) {
        x = __dsub_rn(x, size);
        if (++it > MINIMAGE_MAX_ITERS) return false;
    }
    while (x < -radius) {
        x = __dadd_rn(x, size);
        if (++it > MINIMAGE_MAX_ITERS) return false;
    }
    return true;
}

__device__ __forceinline__ bool wrap_periodic64(double& x, double lo, double hi)
{
    int it = 0;
    double w = __dsub_rn(hi, lo);
    while (x < lo) {
        x = __dadd_rn(x, w);
        if (++it > MINIMAGE_MAX_ITERS) return false;
    }
    while (x >= hi) {
        x = __dsub_rn(x, w);
        if (++it > MINIMAGE_MAX_ITERS) return false;
    }
    return true;
}

// CG: load the positions through L2 (__ldcg), for kernels whose other blocks
// wrote them earlier in the same launch.
template <bool CG = false>
__device__ __forceinline__ bool distance64(const double* xi, const double* xj, int bc, const RepDev& R, Dist64& o)
{
    double x = __dsub_rn(CG ? __ldcg(xi) : xi[0], CG ? __ldcg(xj) : xj[0]);
    double y = __dsub_rn(CG ? __ldcg(xi + 1) : xi[1], CG ? __ldcg(xj + 1) : xj[1]);
    double z = __dsub_rn(CG ? __ldcg(xi + 2) : xi[2], CG ? __ldcg(xj + 2) : xj[2]);
    bool ok = true;
    if (bc == NBG_BC_CUBIC) {
        double size = R.L;
        double radius = __dmul_rn(0.5, size);
        ok = wrap_cubic64(x, size, radius) && wrap_cubic64(y, size, radius) && wrap_cubic64(z, size, radius);
    } else if (bc == NBG_BC_PERIODIC) {
        ok = wrap_periodic64(x, R.box[0], R.box[1]) && wrap_periodic64(y, R.box[2], R.box[3]) &&
             wrap_periodic64(z, R.box[4], R.box[5]);
    }
    o.x = x;
    o.y = y;
    o.z = z;
    o.r2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
    return ok;
}

// The FP32 constants of a replica's pair test, copied into registers before
// a pair loop (read through a reference to the replica table they would be
// loaded again for every pair).
struct PairK {
    float invLf, Lh, Ll, lj_lo, lj_hi, el_lo, el_hi;
    __device__ __forceinline__ explicit PairK(const RepDev& R)
        : invLf(R.invLf), Lh(R.Lh), Ll(R.Ll), lj_lo(R.lj_lo), lj_hi(R.lj_hi), el_lo(R.el_lo), el_hi(R.el_hi)
    {
    }
};

// FP32 difference of two split positions; under cubic boundaries the hi
// parts are exact multiples of the grid and the image shift is exact.
// R: a RepDev or a PairK (invLf, Lh, Ll).
template <class P>
__device__ __forceinline__ float3 split_diff(const float4& hi_i, const float4& lo_i, const float4& hi_j,
                                             const float4& lo_j, bool cubic, const P& R)
{
    float dxh = __fsub_rn(hi_i.x, hi_j.x);
    float dyh = __fsub_rn(hi_i.y, hi_j.y);
    float dzh = __fsub_rn(hi_i.z, hi_j.z);
    float dxl = __fsub_rn(lo_i.x, lo_j.x);
    float dyl = __fsub_rn(lo_i.y, lo_j.y);
    float dzl = __fsub_rn(lo_i.z, lo_j.z);
    if (cubic) {
        // s = rint(dh / L) by the 1.5 * 2^23 trick, exact for |dh/L| <= 1
        const float magic = 12582912.0f;
        float sx = __fsub_rn(__fmaf_rn(dxh, R.invLf, magic), magic);
        float sy = __fsub_rn(__fmaf_rn(dyh, R.invLf, magic), magic);
        float sz = __fsub_rn(__fmaf_rn(dzh, R.invLf, magic), magic);
        dxh = __fmaf_rn(-sx, R.Lh, dxh);
        dyh = __fmaf_rn(-sy, R.Lh, dyh);
        dzh = __fmaf_rn(-sz, R.Lh, dzh);
        dxl = __fmaf_rn(-sx, R.Ll, dxl);
        dyl = __fmaf_rn(-sy, R.Ll, dyl);
        dzl = __fmaf_rn(-sz, R.Ll, dzl);
    }
    return make_float3(__fadd_rn(dxh, dxl), __fadd_rn(dyh, dyl), __fadd_rn(dzh, dzl));
}

// Electrostatic exclusion: self, or the same molecule for water
// (nbody_to_ode.jl:316-351).
__device__ __forceinline__ bool el_excluded(int kind, int64_t i, int64_t j)
{
    return kind == NBG_SYSTEM_WATER ? (i / 3 == j / 3) : (i == j);
}

// Result of classifying and evaluating one ordered pair (i, j).
struct PairOut {
    float fx, fy, fz;   // force contribution (already scaled by 24 eps / k q_i)
    int lj_in, el_in;
    bool range_err;
};

// One ordered pair of the cutoff potentials (LJ basic_potentials.jl:253-265,
// electrostatics :288-297 generalised to reaction field). Classification:
// FP32 r^2 decides clear cases, pairs within CLASSIFY_MARGIN of a cutoff (or
// near the half-box image ambiguity) are decided by the reference's FP64
// arithmetic on the unwrapped positions, so the pair set equals the
// reference's bit for bit.
// K: the FP32 pair constants, a PairK in registers or the RepDev itself
// (fewer registers; the lanes-per-atom kernel keeps more warps resident so)
template <bool CG = false, class KT = PairK>
__device__ __forceinline__ PairOut pair_cutoff(const Dev& d, const RepDev& R, const KT& K, int64_t i, int64_t j,
                                               const float4& hi_i, const float4& lo_i, const float4& hi_j,
                                               const float4& lo_j, float kqi, const double* X)
{
    PairOut o;
    o.fx = o.fy = o.fz = 0.0f;
    o.lj_in = o.el_in = 0;
    o.range_err = false;
    const bool cubic = d.bc == NBG_BC_CUBIC;
    float3 dr = split_diff(hi_i, lo_i, hi_j, lo_j, cubic, K);
    float r2 = __fmaf_rn(dr.x, dr.x, __fmaf_rn(dr.y, dr.y, __fmul_rn(dr.z, dr.z)));
    const bool lj_pair = (d.pots & NBG_POT_LJ) && ((__float_as_int(lo_i.w) & __float_as_int(lo_j.w) & AF_LJ) != 0);
    const bool el_pair = (d.pots & NBG_POT_EL) && !el_excluded(d.kind, i, j);
    bool amb = false;
    if (lj_pair) {
        if (r2 < K.lj_lo) o.lj_in = 1;
        else if (r2 < K.lj_hi) amb = true;
    }
    if (el_pair) {
        if (r2 < K.el_lo) o.el_in = 1;
        else if (r2 < K.el_hi) amb = true;
    }
    if (amb || d.bc == NBG_BC_PERIODIC) {
        Dist64 q;
        bool ok = distance64<CG>(X + 3 * i, X + 3 * j, d.bc, R, q);
        if (!ok) {
            o.range_err = true;
            o.lj_in = o.el_in = 0;
            return o;
        }
        o.lj_in = lj_pair && (q.r2 < d.lj_R2);
        o.el_in = el_pair && (q.r2 < d.el_R2);
        dr = make_float3((float)q.x, (float)q.y, (float)q.z);
        r2 = (float)q.r2;
    }
    float factor = 0.0f;
    if (o.lj_in) {
        float s6 = __fdividef(d.lj_sig2, r2);
        s6 = s6 * s6 * s6;
        float s12 = s6 * s6;
        factor = d.lj_eps24 * __fdividef(2.0f * s12 - s6, r2);
    }
    if (o.el_in) {
        float rinv = rsqrtf(r2);
        // reaction field: q_j (1/r^3 - 2 k_rf); k_rf = 0 for eps_rf = 1
        factor += kqi * hi_j.w * (rinv * rinv * rinv - d.el_krf2);
    }
    o.fx = factor * dr.x;
    o.fy = factor * dr.y;
    o.fz = factor * dr.z;
    return o;
}

// Split a position into (hi, lo) floats (see the layout note above).
__device__ __forceinline__ void split_position(const Dev& d, const RepDev& R, const double* p, float* h, float* l)
{
    if (d.bc == NBG_BC_CUBIC) {
        for (int k = 0; k < 3; ++k) {
            double w = p[k] - R.L * floor(p[k] * R.invL);
            if (w < 0.0) w += R.L;
            if (w >= R.L) w -= R.L;
            double hq = rint(w * (double)R.qscale) * (double)R.qinv;
            h[k] = (float)hq;
            l[k] = (float)(w - hq);
        }
    } else {
        for (int k = 0; k < 3; ++k) {
            h[k] = (float)p[k];
            l[k] = (float)(p[k] - (double)h[k]);
        }
    }
}

// Split of a position shifted by a given periodic image, w = p - L img:
// between list builds (img fixed at the build) w stays within skin/2 of the
// box, well inside the exact range of the hi grid (|w| < 4 L).
__device__ __forceinline__ void split_position_image(const RepDev& R, const double* p, const double* img, float* h,
                                                     float* l)
{
    for (int k = 0; k < 3; ++k) {
        const double w = fma(-R.L, img[k], p[k]);
        const double hq = rint(w * (double)R.qscale) * (double)R.qinv;
        h[k] = (float)hq;
        l[k] = (float)(w - hq);
    }
}

// Fixed-point box coordinate: x / L * 2^32 rounded, modulo 2^32 (the wrap
// into the box is the integer truncation; exact to 2^-21 of a unit for
// positions within 1024 boxes of the origin).
__device__ __forceinline__ unsigned fx_coord(double x, double scale)
{
    return (unsigned)(unsigned long long)__double2ll_rn(__dmul_rn(x, scale));
}

__device__ __forceinline__ void pack_fx(const Dev& d, const RepDev& R, int64_t i, const double* X)
{
    uint4 q;
    q.x = fx_coord(X[3 * i], R.fx_scale);
    q.y = fx_coord(X[3 * i + 1], R.fx_scale);
    q.z = fx_coord(X[3 * i + 2], R.fx_scale);
    q.w = d.pfx[i].w;
    d.pfx[i] = q;
}

// ALL: refresh every position form (on-demand evaluations); otherwise the
// steps write the fixed-point form and the split form only when its per-step
// readers run (split_on).
template <bool ALL = false>
__device__ __forceinline__ void pack_atom(const Dev& d, int64_t i, const double* X)
{
    const RepDev& R = d.reps[d.rep_of[i]];
    if (d.pfx) pack_fx(d, R, i, X);
    if (!ALL && !d.split_on) return;
    const double p[3] = {X[3 * i], X[3 * i + 1], X[3 * i + 2]};
    float h[3], l[3];
    if (d.img && d.bc == NBG_BC_CUBIC) split_position_image(R, p, d.img + 3 * i, h, l);
    else split_position(d, R, p, h, l);
    float4 hi = d.phi[i];
    float4 lo = d.plo[i];
    d.phi[i] = make_float4(h[0], h[1], h[2], hi.w);
    d.plo[i] = make_float4(l[0], l[1], l[2], lo.w);
}

// Velocity-Verlet drift of one component, u' = u + dt v + dt^2 (a/2), with
// no contracted multiply-add (the reference's arithmetic).
__device__ __forceinline__ double drift1(double u, double v, double a, double dt, double dtsq)
{
    return __dadd_rn(__dadd_rn(u, __dmul_rn(dt, v)), __dmul_rn(dtsq, __dmul_rn(0.5, a)));
}

// Velocity-Verlet kick of one component, v' = v + dt (a/2 + a'/2).
__device__ __forceinline__ double kick1(double v, double a, double an, double dt)
{
    return __dadd_rn(v, __dmul_rn(dt, __dadd_rn(__dmul_rn(0.5, a), __dmul_rn(0.5, an))));
}

// TwoSum: s + e = a + b exactly (Knuth).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Accumulator of float partials with a compensated (hi, lo) pair.
struct Acc2 {
    float hi, lo;
    __device__ __forceinline__ void add(float p)
    {
        float s, e;
        two_sum(hi, p, s, e);
        hi = s;
        lo = __fadd_rn(lo, e);
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// Philox4x32-10 (Salmon et al., SC'11); counter (atom, step lo, step hi, stream)
__device__ __forceinline__ uint4 philox(uint64_t seed, uint64_t atom, uint64_t step, uint32_t stream)
{
    uint32_t c0 = (uint32_t)atom, c1 = (uint32_t)step, c2 = (uint32_t)(step >> 32), c3 = stream;
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return make_uint4(c0, c1, c2, c3);
}

__device__ __forceinline__ double philox_u53(uint64_t seed, uint64_t atom, uint64_t step)
{
    uint4 w = philox(seed, atom, step, 0u);
    return ((double)(w.x >> 5) * 67108864.0 + (double)(w.y >> 6)) * (1.0 / 9007199254740992.0);
}

// Three normals from 24-bit uniforms (same draws as the oracle's).
template <typename T>
__device__ __forceinline__ void philox_normals3(uint64_t seed, uint64_t atom, uint64_t step, T out[3])
{
    uint4 w1 = philox(seed, atom, step, 1u);
    uint4 w2 = philox(seed, atom, step, 2u);
    const T two_pi = (T)6.283185307179586;
    const T s24 = (T)(1.0 / 16777216.0);
    T u1 = ((T)(w1.x >> 8) + (T)1) * s24;
    T u2 = (T)(w1.y >> 8) * s24;
    T rr = sqrt((T)-2 * log(u1));
    T sn, cs;
    sincos(two_pi * u2, &sn, &cs);
    out[0] = rr * cs;
    out[1] = rr * sn;
    T u3 = ((T)(w2.x >> 8) + (T)1) * s24;
    T u4 = (T)(w2.y >> 8) * s24;
    out[2] = sqrt((T)-2 * log(u3)) * cos(two_pi * u4);
}

#endif  // __CUDACC__
