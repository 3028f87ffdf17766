// nbg_api.cu - the C ABI of include/nbg.h: context lifecycle, marshalling of
// the system descriptor into device buffers, and the step loops.
//
// Step loops (all work asynchronous on the context's stream):
//   velocity Verlet  drift -> [Verlet list] -> forces -> [bonded] ->
//                    [temperature] -> kick -> [Andersen]
//   Euler-Maruyama   [Verlet list] -> forces -> [bonded] -> EM update
// nbg_advance runs the loop in chunks; after each chunk it reads the device
// status word. A cell or neighbour capacity overflow restores the chunk's
// starting state, grows the capacity and runs the chunk again; non-finite
// accelerations or a minimum-image loop over its iteration cap end the call
// with an error.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "nbg_internal.cuh"

static const char* kVersion = "libnbg 1.0 (sm_103a)";

int cuda_fail(nbg_ctx* c, cudaError_t e, const char* what)
{
    if (c) c->err = std::string(what) + ": " + cudaGetErrorString(e);
    return NBG_ERR_CUDA;
}

static int fail(nbg_ctx* c, int code, const std::string& msg)
{
    if (c) c->err = msg;
    return code;
}

#define CK(call, what)                                        \
    do {                                                      \
        cudaError_t _e = (call);                              \
        if (_e != cudaSuccess) return cuda_fail(c, _e, what); \
    } while (0)

static int plan_cluster(nbg_ctx* c);
static int settle(nbg_ctx* c);
// entry of a context call: the device current, any deferred step status read
#define NBG_ENTER(c)                           \
    do {                                       \
        cudaSetDevice((c)->device);            \
        int _settled = settle(c);              \
        if (_settled) return _settled;         \
    } while (0)

template <typename T>
static int dalloc(nbg_ctx* c, T** p, size_t count)
{
    void* q = nullptr;
    size_t bytes = count * sizeof(T);
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(c, NBG_ERR_NOMEM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
    }
    cudaMemset(q, 0, bytes);
    c->allocs.push_back(q);
    *p = (T*)q;
    return NBG_OK;
}

static void dfree(nbg_ctx* c, void* p)
{
    if (!p) return;
    auto it = std::find(c->allocs.begin(), c->allocs.end(), p);
    if (it != c->allocs.end()) c->allocs.erase(it);
    cudaFree(p);
}

extern "C" const char* nbg_version(void) { return kVersion; }
extern "C" int nbg_abi_version(void) { return NBG_ABI_VERSION; }

const char* noalloc_last_error();

extern "C" const char* nbg_last_error(const nbg_ctx* ctx)
{
    if (!ctx) return noalloc_last_error();  // errors of the context-free entry points
    return ctx->err.c_str();
}

extern "C" int64_t nbg_kernel_launches(const nbg_ctx* ctx) { return ctx ? ctx->launches : 0; }

// ---------------------------------------------------------------------
// descriptor validation
// ---------------------------------------------------------------------
static int validate(const nbg_system_desc* d, std::string& why)
{
    if (!d) { why = "null descriptor"; return NBG_ERR_ARG; }
    if (d->abi_version != NBG_ABI_VERSION) { why = "abi_version mismatch"; return NBG_ERR_ARG; }
    if (d->n < 1) { why = "n must be >= 1"; return NBG_ERR_ARG; }
    if (d->n > (1ll << 30)) { why = "n above 2^30 atoms"; return NBG_ERR_UNSUPPORTED; }
    if (!d->mass) { why = "mass is required"; return NBG_ERR_ARG; }
    for (int64_t i = 0; i < d->n; ++i)
        if (!(d->mass[i] > 0.0) || !std::isfinite(d->mass[i])) { why = "masses must be finite and > 0"; return NBG_ERR_ARG; }
    if (d->kind != NBG_SYSTEM_POTENTIAL && d->kind != NBG_SYSTEM_WATER) { why = "unknown system kind"; return NBG_ERR_ARG; }
    uint32_t pots = d->kind == NBG_SYSTEM_WATER ? (NBG_POT_LJ | NBG_POT_EL) : d->potentials;
    if (pots & ~15u) { why = "unknown potential bits"; return NBG_ERR_ARG; }
    if (d->kind == NBG_SYSTEM_WATER && d->n % 3 != 0) { why = "water needs 3 atoms per molecule"; return NBG_ERR_ARG; }
    if ((pots & NBG_POT_EL) && !d->charge) { why = "charges are required"; return NBG_ERR_ARG; }
    if ((pots & NBG_POT_MAG) && !d->dipole) { why = "dipoles are required"; return NBG_ERR_ARG; }
    if ((pots & NBG_POT_LJ) && !(d->lj_cutoff > 0.0)) { why = "LJ cutoff must be > 0"; return NBG_ERR_ARG; }
    if ((pots & NBG_POT_EL) && !(d->el_cutoff > 0.0)) { why = "electrostatic cutoff must be > 0"; return NBG_ERR_ARG; }
    if ((pots & NBG_POT_EL) && !(d->el_eps_rf >= 1.0)) { why = "eps_rf must be >= 1"; return NBG_ERR_ARG; }
    if (d->bc == NBG_BC_CUBIC) {
        if (!(d->box[0] > 0.0) || !std::isfinite(d->box[0])) { why = "cubic box needs finite L > 0"; return NBG_ERR_ARG; }
    } else if (d->bc == NBG_BC_PERIODIC) {
        for (int k = 0; k < 3; ++k)
            if (!(d->box[2 * k + 1] > d->box[2 * k])) { why = "periodic box needs hi > lo"; return NBG_ERR_ARG; }
    } else if (d->bc != NBG_BC_INFINITE) {
        why = "unknown boundary";
        return NBG_ERR_ARG;
    }
    if (d->thermostat < NBG_THERMO_NULL || d->thermostat > NBG_THERMO_LANGEVIN) { why = "unknown thermostat"; return NBG_ERR_ARG; }
    if (d->thermostat != NBG_THERMO_NULL) {
        if (!(d->thermo_param > 0.0)) { why = "thermostat parameter must be > 0"; return NBG_ERR_ARG; }
        if (!(d->kb > 0.0)) { why = "kb must be > 0"; return NBG_ERR_ARG; }
    }
    return NBG_OK;
}

// ---------------------------------------------------------------------
// context construction
// ---------------------------------------------------------------------
static float f_down(double x) { float f = (float)x; if ((double)f > x) f = nextafterf(f, 0.0f); return f; }
static float f_up(double x)
{
    if (std::isinf(x)) return INFINITY;
    float f = (float)x;
    if ((double)f < x) f = nextafterf(f, INFINITY);
    return f;
}

static double list_radius(const nbg_system_desc* d)
{
    uint32_t pots = d->kind == NBG_SYSTEM_WATER ? (NBG_POT_LJ | NBG_POT_EL) : d->potentials;
    double rc = 0.0;
    if (pots & NBG_POT_LJ) rc = std::max(rc, d->lj_cutoff);
    if (pots & NBG_POT_EL) rc = std::max(rc, d->el_cutoff);
    return rc + std::max(d->skin, 0.0);
}

static int choose_path(const nbg_system_desc* descs, int nrep)
{
    const nbg_system_desc* d = &descs[0];
    uint32_t pots = d->kind == NBG_SYSTEM_WATER ? (NBG_POT_LJ | NBG_POT_EL) : d->potentials;
    if (nrep == 1 && d->kind == NBG_SYSTEM_POTENTIAL && pots == NBG_POT_GRAV) return PATH_GRAVITY;
    bool list_ok = !(d->flags & NBG_FLAG_ALL_PAIRS) && d->bc == NBG_BC_CUBIC && (pots & ~(uint32_t)(NBG_POT_LJ | NBG_POT_EL)) == 0 &&
                   pots != 0;
    if (list_ok) {
        // a single system needs at least 3 cells per side to gain from cells;
        // a batch keeps small replicas on the list path as one cell each
        for (int r = 0; r < nrep; ++r) {
            double rl = list_radius(&descs[r]);
            if (!std::isfinite(rl)) { list_ok = false; break; }
            int nc = (int)std::floor(descs[r].box[0] / (rl * (1.0 + 1e-4)));
            if (nc < 3 && nrep == 1) { list_ok = false; break; }
        }
    }
    if (list_ok) return PATH_LIST;
    if (nrep == 1) return PATH_ALLPAIRS;
    return -1;
}

// Verlet-list layout of the force kernel's lanes per atom
static void set_list_layout(nbg_ctx* c)
{
    if (c->list_lpa <= 1) {  // column-major for thread per atom
        c->d.nbr_kstride = c->n;
        c->d.nbr_istride = 1;
    } else {                 // row-major for lanes per atom
        c->d.nbr_kstride = 1;
        c->d.nbr_istride = c->d.nbr_cap;
    }
}

// The list force kernel's form for the current lanes per atom and list
// buffer: the fixed-point kernel where it fits, and whether the steps must
// also keep the split positions current (the split-form kernels or the
// learned model read them every step). Captured graphs hold the old form.
static int set_force_form(nbg_ctx* c)
{
    set_list_layout(c);
    int st = fx_prepare(c);
    if (st) return st;
    c->d.split_on = (!c->fx_ready || c->ml_on) ? 1 : 0;
    if (c->graph) {
        cudaGraphExecDestroy(c->graph);
        c->graph = nullptr;
    }
    if (c->accel_graph) {
        cudaGraphExecDestroy(c->accel_graph);
        c->accel_graph = nullptr;
    }
    c->accel_lists_valid = false;
    return NBG_OK;
}

static int alloc_lists(nbg_ctx* c, int cell_cap, int nbr_cap)
{
    int st;
    if (c->d.cell_atoms) dfree(c, c->d.cell_atoms);
    if (c->d.nbr) dfree(c, c->d.nbr);
    c->d.cell_atoms = nullptr;
    c->d.nbr = nullptr;
    if ((st = dalloc(c, &c->d.cell_atoms, (size_t)c->d.ncell_total * cell_cap))) return st;
    if ((st = dalloc(c, &c->d.nbr, (size_t)c->n * nbr_cap))) return st;
    c->d.cell_cap = cell_cap;
    c->d.nbr_cap = nbr_cap;
    return set_force_form(c);
}

static int build_context(nbg_ctx* c, const nbg_system_desc* descs, int nrep)
{
    const nbg_system_desc* d0 = &descs[0];
    // read before the list buffers (and the force kernel's form) are set up
    if (getenv("NBG_FX_BLOCK")) c->fx_block_only = true;  // per-block list staging (comparisons)
    c->desc = *d0;
    c->desc.mass = c->desc.charge = c->desc.dipole = nullptr;
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device);
    if (c->sms < 1) c->sms = 1;
    c->nrep = nrep;
    uint32_t pots = d0->kind == NBG_SYSTEM_WATER ? (NBG_POT_LJ | NBG_POT_EL) : d0->potentials;
    int64_t n = 0;
    for (int r = 0; r < nrep; ++r) n += descs[r].n;
    c->n = n;
    c->cols = n + ((nrep == 1 && d0->thermostat == NBG_THERMO_NOSEHOOVER) ? 1 : 0);
    c->path = choose_path(descs, nrep);
    if (c->path < 0) return fail(c, NBG_ERR_UNSUPPORTED, "a batch needs every replica on the cubic Verlet-list path");

    // per-atom host arrays
    c->mass_h.resize(n);
    c->charge_h.assign(n, 0.0);
    if (pots & NBG_POT_MAG) c->dipole_h.assign(3 * n, 0.0);
    std::vector<int> rep_of(n);
    int64_t off = 0;
    for (int r = 0; r < nrep; ++r) {
        const nbg_system_desc* d = &descs[r];
        for (int64_t i = 0; i < d->n; ++i) {
            c->mass_h[off + i] = d->mass[i];
            if (pots & NBG_POT_EL) c->charge_h[off + i] = d->charge[i];
            if (pots & NBG_POT_MAG)
                for (int k = 0; k < 3; ++k) c->dipole_h[3 * (off + i) + k] = d->dipole[3 * i + k];
            rep_of[off + i] = r;
        }
        off += d->n;
    }

    Dev& D = c->d;
    D.n = n;
    D.cols = c->cols;
    D.kind = d0->kind;
    D.bc = d0->bc;
    D.therm = d0->thermostat;
    D.nrep = nrep;
    D.pots = pots;
    D.lj_sig2_d = d0->lj_sigma * d0->lj_sigma;
    D.lj_sig2 = (float)D.lj_sig2_d;
    D.lj_eps = d0->lj_epsilon;
    D.lj_eps24 = (float)(24.0 * d0->lj_epsilon);
    D.lj_R2 = d0->lj_cutoff * d0->lj_cutoff;
    D.el_k_d = d0->el_k;
    D.el_k = (float)d0->el_k;
    D.el_R = d0->el_cutoff;
    D.el_R2 = d0->el_cutoff * d0->el_cutoff;
    // reaction field with a vacuum (eps = 1) inside the cutoff
    double eps_rf = d0->el_eps_rf;
    if (std::isfinite(d0->el_cutoff) && eps_rf != 1.0) {
        double R3 = d0->el_cutoff * d0->el_cutoff * d0->el_cutoff;
        D.el_krf = std::isinf(eps_rf) ? 0.5 / R3 : (eps_rf - 1.0) / ((2.0 * eps_rf + 1.0) * R3);
        D.el_crf = 1.0 / d0->el_cutoff + D.el_krf * d0->el_cutoff * d0->el_cutoff;
    } else {
        D.el_krf = 0.0;
        D.el_crf = std::isfinite(d0->el_cutoff) ? 1.0 / d0->el_cutoff : 0.0;
    }
    D.el_krf2 = (float)(2.0 * D.el_krf);
    D.split_on = 1;
    D.G = d0->grav_G;
    D.mu4pi = d0->mag_mu_4pi;
    D.kb = d0->kb;
    D.rOH = d0->water_rOH;
    D.aHOH = d0->water_aHOH;
    D.kbond = d0->water_kb;
    D.kangle = d0->water_ka;
    D.skin_half2 = 0.25 * std::max(d0->skin, 0.0) * std::max(d0->skin, 0.0);
    D.grav_plain = (d0->flags & NBG_FLAG_GRAV_PLAIN) ? 1 : 0;
    c->baoab = d0->thermostat == NBG_THERMO_LANGEVIN && (d0->flags & NBG_FLAG_LANGEVIN_BAOAB);

    // replicas
    c->reps_h.resize(nrep);
    off = 0;
    int cell0 = 0;
    int max_cell_occ = 0;
    double max_nbr = 0.0;
    int64_t max_rep_n = 0;
    for (int r = 0; r < nrep; ++r) {
        const nbg_system_desc* d = &descs[r];
        RepDev R{};
        R.atom0 = off;
        R.n = d->n;
        max_rep_n = std::max(max_rep_n, d->n);
        for (int k = 0; k < 6; ++k) R.box[k] = d->box[k];
        double img2 = INFINITY;
        if (d->bc == NBG_BC_CUBIC) {
            double L = d->box[0];
            R.L = L;
            R.invL = 1.0 / L;
            int e = (int)std::ceil(std::log2(L));
            int k = 22 - e;
            R.qscale = (float)std::ldexp(1.0, k);
            R.qinv = (float)std::ldexp(1.0, -k);
            double Lh = std::rint(L * std::ldexp(1.0, k)) * std::ldexp(1.0, -k);
            R.Lh = (float)Lh;
            R.Ll = (float)(L - Lh);
            R.invLf = (float)(1.0 / L);
            double h = 0.5 * L * (1.0 - CLASSIFY_MARGIN);
            img2 = h * h;
        }
        double m = CLASSIFY_MARGIN;
        if (pots & NBG_POT_LJ) {
            double R2 = d0->lj_cutoff * d0->lj_cutoff;
            R.lj_lo = f_down(std::min(R2 * (1.0 - m), img2));
            R.lj_hi = f_up(R2 * (1.0 + m));
        }
        if (pots & NBG_POT_EL) {
            double R2 = d0->el_cutoff * d0->el_cutoff;
            R.el_lo = f_down(std::min(R2 * (1.0 - m), img2));
            R.el_hi = f_up(R2 * (1.0 + m));
        }
        if (d->bc == NBG_BC_CUBIC) {
            // fixed-point box units u = L / 2^32 (the same bands, in u^2)
            const double L = d->box[0];
            const double u = L / 4294967296.0, iu2 = 1.0 / (u * u);
            R.fx_scale = 4294967296.0 / L;
            const double hb = 2147483648.0 * (1.0 - m), img2b = hb * hb;
            R.fx_fscale = (pots & NBG_POT_LJ) ? 24.0 * d0->lj_epsilon / u : 1.0;
            R.fx_kq = D.el_k_d * (R.fx_scale * R.fx_scale) / R.fx_fscale;
            if (pots & NBG_POT_LJ) {
                const double R2 = d0->lj_cutoff * d0->lj_cutoff * iu2;
                R.fx_lj_lo = f_down(std::min(R2 * (1.0 - m), img2b));
                R.fx_lj_hi = f_up(R2 * (1.0 + m));
                const double s2 = d0->lj_sigma * d0->lj_sigma * iu2;
                R.fx_sig2_hi = (float)s2;
                R.fx_sig2_lo = (float)(s2 - (double)R.fx_sig2_hi);
            }
            const double rlb = list_radius(d);
            R.fx_rl2 = f_up(rlb * rlb * (1.0 + 1e-5) * iu2);
            const double sh = 0.5 * std::max(d->skin, 0.0);
            R.fx_disp2 = f_down(sh * sh * iu2 * (1.0 - 1e-4));
            if (pots & NBG_POT_EL) {
                const double R2 = d0->el_cutoff * d0->el_cutoff * iu2;
                R.fx_el_lo = f_down(std::min(R2 * (1.0 - m), img2b));
                R.fx_el_hi = f_up(R2 * (1.0 + m));
                R.fx_krf = (float)(2.0 * D.el_krf * u * u * u);
            }
        }
        if (c->path == PATH_LIST) {
            double rl = list_radius(d);
            // cells of at least rl / 2 scanned over a 5 x 5 x 5 stencil (2.4x fewer
            // candidates than rl cells over 3 x 3 x 3) when the box holds 5 per side
            // and a half cell holds 16 atoms on average (below that the per-cell
            // work of the builders dominates), else cells of rl over 3 x 3 x 3,
            // else one cell for the replica
            const int nc2 = (int)std::floor(d->box[0] / (0.5 * rl * (1.0 + 1e-4)));
            const int nc1 = (int)std::floor(d->box[0] / (rl * (1.0 + 1e-4)));
            const double occ2 = nc2 > 0 ? (double)d->n / ((double)nc2 * nc2 * nc2) : 0.0;
            if (nc2 >= 5 && occ2 >= 16.0) {
                R.nc = nc2;
                R.ns = 2;
            } else if (nc1 >= 3) {
                R.nc = nc1;
                R.ns = 1;
            } else {
                R.nc = 1;  // one cell holding the whole replica
                R.ns = 0;
            }
            R.cell0 = cell0;
            R.cell_inv = R.nc / d->box[0];
            R.rl2 = f_up(rl * rl * (1.0 + 1e-5));
            cell0 += R.nc * R.nc * R.nc;
            double rho = d->n / (d->box[0] * d->box[0] * d->box[0]);
            double cs = d->box[0] / R.nc;
            max_cell_occ = std::max(max_cell_occ, (int)std::ceil(rho * cs * cs * cs));
            max_nbr = std::max(max_nbr, 4.0 / 3.0 * M_PI * rl * rl * rl * rho);
        }
        R.T0 = d->thermo_T;
        R.tparam = d->thermo_param;
        if (d->thermostat == NBG_THERMO_LANGEVIN) {
            R.sigma = std::sqrt(2.0 * d->thermo_param * d->kb * d->thermo_T / d->mass[0]);
            R.sigma_num = std::sqrt(2.0 * d->thermo_param * d->kb * d->thermo_T);
        }
        int64_t Nc = d->kind == NBG_SYSTEM_WATER ? 2 * (d->n / 3) : 0;
        R.ndf = (double)(3 * d->n - Nc);
        R.seed = d->seed;
        c->reps_h[r] = R;
        off += d->n;
    }
    D.ncell_total = cell0;

    int st;
    {
        std::vector<int> cr((size_t)std::max(cell0, 1), 0);
        for (int r = 0; r < nrep; ++r) {
            const RepDev& R = c->reps_h[r];
            if (c->path != PATH_LIST) break;
            for (int k = 0; k < R.nc * R.nc * R.nc; ++k) cr[(size_t)R.cell0 + k] = r;
        }
        int* cp = nullptr;
        if ((st = dalloc(c, &cp, cr.size()))) return st;
        CK(cudaMemcpy(cp, cr.data(), sizeof(int) * cr.size(), cudaMemcpyHostToDevice), "cell_rep upload");
        D.cell_rep = cp;
    }
    // state
    StateView* views[2] = {&c->st, &c->ev};
    for (StateView* sv : views) {
        double* blk = nullptr;  // x, v, a_old, a_new in one allocation (one-copy backups)
        if ((st = dalloc(c, &blk, 12 * (size_t)c->cols))) return st;
        sv->x = blk;
        sv->v = blk + 3 * c->cols;
        sv->a_old = blk + 6 * c->cols;
        sv->a_new = blk + 9 * c->cols;
    }
    // gravity bodies padded to a multiple of the largest i-block (4 x 128)
    c->npad = c->path == PATH_GRAVITY ? ((n + 511) / 512) * 512 : n;
    double* dp;
    if ((st = dalloc(c, &dp, n))) return st;
    D.mass = dp;
    CK(cudaMemcpy(dp, c->mass_h.data(), sizeof(double) * n, cudaMemcpyHostToDevice), "mass upload");
    std::vector<double> im(n);
    for (int64_t i = 0; i < n; ++i) im[i] = 1.0 / c->mass_h[i];
    if ((st = dalloc(c, &dp, n))) return st;
    D.inv_mass = dp;
    CK(cudaMemcpy(dp, im.data(), sizeof(double) * n, cudaMemcpyHostToDevice), "inv_mass upload");
    {
        std::vector<double> rs(n);
        for (int64_t i = 0; i < n; ++i) rs[i] = std::sqrt(im[i]);
        double* rp = nullptr;
        if ((st = dalloc(c, &rp, n))) return st;
        D.rsqrt_mass = rp;
        CK(cudaMemcpy(rp, rs.data(), sizeof(double) * n, cudaMemcpyHostToDevice), "rsqrt_mass upload");
    }
    if ((st = dalloc(c, &dp, n))) return st;
    D.charge = dp;
    CK(cudaMemcpy(dp, c->charge_h.data(), sizeof(double) * n, cudaMemcpyHostToDevice), "charge upload");
    if (pots & NBG_POT_MAG) {
        if ((st = dalloc(c, &dp, 3 * n))) return st;
        D.dipole = dp;
        CK(cudaMemcpy(dp, c->dipole_h.data(), sizeof(double) * 3 * n, cudaMemcpyHostToDevice), "dipole upload");
    }
    int* ip;
    if ((st = dalloc(c, &ip, n))) return st;
    D.rep_of = ip;
    CK(cudaMemcpy(ip, rep_of.data(), sizeof(int) * n, cudaMemcpyHostToDevice), "rep_of upload");
    RepDev* rp;
    if ((st = dalloc(c, &rp, nrep))) return st;
    D.reps = rp;
    CK(cudaMemcpy(rp, c->reps_h.data(), sizeof(RepDev) * nrep, cudaMemcpyHostToDevice), "replica upload");

    // split positions with their static w (charge or mass) and flags
    if ((st = dalloc(c, &D.phi, c->npad))) return st;
    if ((st = dalloc(c, &D.plo, c->npad))) return st;
    {
        std::vector<float4> hi(c->npad), lo(c->npad);
        for (int64_t i = 0; i < c->npad; ++i) {
            if (i >= n) {  // padding body: far away, massless
                hi[i] = make_float4(1e18f, 1e18f, 1e18f, 0.0f);
                lo[i] = make_float4(0.f, 0.f, 0.f, 0.f);
                continue;
            }
            float w = c->path == PATH_GRAVITY ? (float)c->mass_h[i] : (float)c->charge_h[i];
            int flags = 0;
            int64_t li = i - c->reps_h[rep_of[i]].atom0;
            if ((pots & NBG_POT_LJ) && (d0->kind != NBG_SYSTEM_WATER || li % 3 == 0)) flags |= AF_LJ;
            hi[i] = make_float4(0.f, 0.f, 0.f, w);
            float wf;
            memcpy(&wf, &flags, sizeof(float));
            lo[i] = make_float4(0.f, 0.f, 0.f, wf);
        }
        CK(cudaMemcpy(D.phi, hi.data(), sizeof(float4) * c->npad, cudaMemcpyHostToDevice), "phi init");
        CK(cudaMemcpy(D.plo, lo.data(), sizeof(float4) * c->npad, cudaMemcpyHostToDevice), "plo init");
    }

    if ((st = dalloc(c, &D.status, 4))) return st;
    if ((st = dalloc(c, &D.rebuild_flag, 2 * (size_t)nrep))) return st;
    if ((st = dalloc(c, &D.build_count, 1))) return st;
    if ((st = dalloc(c, &D.step_dev, 1))) return st;
    if ((st = dalloc(c, &D.sink, 1))) return st;  // zeroed: every = 0, nothing saved
    // slices of 256 atoms per replica (the last block adds them in order)
    D.red_slices = (int)std::min<int64_t>(512, std::max<int64_t>(1, (max_rep_n + 255) / 256));
    if ((st = dalloc(c, &D.red_partial, (size_t)nrep * D.red_slices))) return st;
    if ((st = dalloc(c, &D.red_T, nrep))) return st;
    if ((st = dalloc(c, &D.red_counter, nrep))) return st;
    c->kick_blocks = (int)std::min<int64_t>(4096, std::max<int64_t>(1, (3 * n + 255) / 256));
    if ((st = dalloc(c, &c->kick_part, c->kick_blocks))) return st;
    if ((st = dalloc(c, &c->kick_counter, 1))) return st;

    if (c->path == PATH_LIST) {
        // fixed-point positions, w = the FP32 charge (static)
        if (n < ((int64_t)1 << 31) && !getenv("NBG_NO_FX")) {
            if ((st = dalloc(c, &D.pfx, n))) return st;
            std::vector<uint4> q(n);
            for (int64_t i = 0; i < n; ++i) {
                const float qf = (float)c->charge_h[i];
                uint32_t w;
                memcpy(&w, &qf, sizeof w);
                q[i] = make_uint4(0u, 0u, 0u, w);
            }
            CK(cudaMemcpy(D.pfx, q.data(), sizeof(uint4) * n, cudaMemcpyHostToDevice), "pfx init");
        } else {
            c->fx_disabled = true;
        }
        if ((st = dalloc(c, &D.cell_count, D.ncell_total))) return st;
        if ((st = dalloc(c, &D.cell_n, D.ncell_total))) return st;
        if ((st = dalloc(c, &D.nbr_count, n))) return st;
        if ((st = dalloc(c, &D.xref, 3 * n))) return st;
        if (d0->bc == NBG_BC_CUBIC && (st = dalloc(c, &D.img, 3 * n))) return st;
        int cell_cap = ((2 * max_cell_occ + 16 + 7) / 8) * 8;
        int nbr_cap = ((int)std::ceil(1.3 * max_nbr + 32) + 7) / 8 * 8;
        // lanes per atom of the list force kernel: a group of lanes per atom
        // until the GPU holds ~64 resident lanes per SM-thread slot, then one
        // thread per atom (column-major list); and at least one lane per 32
        // list entries (long water lists, as the autotuner finds)
        const char* lv = getenv("NBG_LIST_LPA");  // override for tuning sweeps
        if (lv) {
            c->list_lpa = atoi(lv);
        } else {
            int sms = 0;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
            double threads_wanted = (double)std::max(sms, 1) * 2048.0;
            int lpa = 1;
            while (lpa < 32 && (double)n * lpa < threads_wanted && lpa * 4 <= max_nbr) lpa *= 2;
            while (lpa < 32 && lpa * 32 < max_nbr) lpa *= 2;
            c->list_lpa = lpa;
        }
        // supported group sizes: 1 (thread per atom), 4, 8, 16, 32
        if (c->list_lpa <= 1) c->list_lpa = 1;
        else if (c->list_lpa <= 4) c->list_lpa = 4;
        else if (c->list_lpa <= 8) c->list_lpa = 8;
        else if (c->list_lpa <= 16) c->list_lpa = 16;
        else c->list_lpa = 32;
        if ((st = alloc_lists(c, cell_cap, nbr_cap))) return st;
    }
    if (c->path == PATH_LIST && nrep == 1) {
        // constants of the list-based energy (pairs beyond the cutoffs)
        const bool water = d0->kind == NBG_SYSTEM_WATER;
        const int64_t nlj = water ? n / 3 : n;
        c->lj_pairs = (pots & NBG_POT_LJ) ? nlj * (nlj - 1) / 2 : 0;
        if (pots & NBG_POT_EL) {
            // sum_{i<j} q_i q_j = ((sum q)^2 - sum q^2) / 2, less the intramolecular pairs of water
            long double sq = 0.0L, sq2 = 0.0L, excl = 0.0L;
            for (int64_t i = 0; i < n; ++i) {
                sq += c->charge_h[i];
                sq2 += (long double)c->charge_h[i] * c->charge_h[i];
            }
            if (water)
                for (int64_t m = 0; m + 2 < n; m += 3) {
                    const long double a = c->charge_h[m], b = c->charge_h[m + 1], e = c->charge_h[m + 2];
                    excl += a * b + a * e + b * e;
                }
            c->el_pair_qq = (double)((sq * sq - sq2) / 2.0L - excl);
        }
    }
    if (getenv("NBG_NO_GRAPHS")) c->use_graphs = false;  // direct launches, for comparisons
    if (getenv("NBG_NO_CLUSTER")) c->cluster_disabled = true;  // the graph step loop for small systems too
    // a test of the cluster loop's bounded waits: one launch (the first, or
    // the one after ":k" more) drops the position copies of one step ("last"
    // or a step index), so that the receivers' waits run out with no copy in
    // flight
    if (const char* td = getenv("NBG_TEST_CLUSTER_DROP")) {
        c->cluster_test_drop = strncmp(td, "last", 4) == 0 ? -1 : std::max(0, atoi(td));
        if (const char* k = strchr(td, ':')) c->cluster_test_skip = std::max(0, atoi(k + 1));
    }
#ifdef NBG_DEBUG
    if (const char* pv = getenv("NBG_TEST_PLANT_INDEX")) c->plant_index = std::max(1, atoi(pv));
#endif
    if ((st = plan_cluster(c))) return st;
    if (getenv("NBG_NO_ENSEMBLE_LOOP")) c->ens_disabled = true;  // batches on the step graphs (comparisons)
    if (ensemble_plan(c)) {
        std::vector<int> ord(nrep);
        for (int r = 0; r < nrep; ++r) ord[r] = r;
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return c->reps_h[a].n > c->reps_h[b].n; });
        if ((st = dalloc(c, &c->ens_order, nrep))) return st;
        CK(cudaMemcpy(c->ens_order, ord.data(), sizeof(int) * nrep, cudaMemcpyHostToDevice), "replica order");
        if ((st = dalloc(c, &c->ens_since, nrep))) return st;
        if ((st = dalloc(c, &c->ens_pref, n))) return st;
    }
    if (c->path == PATH_GRAVITY) {
        const char* gv = getenv("NBG_GRAVITY_VARIANT");  // kernel-form override for tuning sweeps
        if (gv) c->grav_variant = atoi(gv);
        const char* gf = getenv("NBG_GRAVITY_FAR_FACTOR");  // far-criterion override for accuracy sweeps
        if (gf && atof(gf) > 0.0) c->grav_far2 = (float)(atof(gf) * atof(gf));
        // equal masses (the Plummer workloads): the mass leaves the pair loop
        // (NBG_GRAVITY_MASSES keeps m_j in the loop, for comparisons)
        c->grav_m0 = c->mass_h[0];
        c->grav_uniform = std::isfinite(c->grav_m0) && c->grav_m0 > 0.0 && !getenv("NBG_GRAVITY_MASSES");
        for (int64_t i = 1; i < n && c->grav_uniform; ++i) c->grav_uniform = c->mass_h[i] == c->grav_m0;
        c->grav_chunks = gravity_plan_chunks(c, c->npad);
        if ((st = dalloc(c, &c->grav_part, (size_t)c->grav_chunks * 3 * n))) return st;
        if (!c->d.grav_plain && !getenv("NBG_GRAVITY_NO_SORT")) {
            c->grav_sort = true;
            for (int k = 0; k < 2; ++k) {
                if ((st = dalloc(c, &c->grav_keys[k], n))) return st;
                if ((st = dalloc(c, &c->grav_vals[k], n))) return st;
            }
            c->grav_sort_bytes = gravity_sort_bytes(n);
            unsigned char* tmp = nullptr;
            if ((st = dalloc(c, &tmp, c->grav_sort_bytes))) return st;
            c->grav_sort_tmp = tmp;
            if ((st = dalloc(c, &c->grav_box, 2 * (c->npad / 128)))) return st;
            if ((st = dalloc(c, &c->grav_extent, 1))) return st;
        }
    }
    return NBG_OK;
}

// The persistent cluster step loop for small systems (k_cluster.cu), if the
// system qualifies at the current list capacity; its FP64 position copies.
static int plan_cluster(nbg_ctx* c)
{
    c->cluster_lists_valid = false;
    c->ens_lists_valid = false;
    c->cla_valid = false;
    if (!cluster_plan(c)) return NBG_OK;
    int st;
    if (!c->cluster_x && (st = dalloc(c, &c->cluster_x, 6 * (size_t)c->n))) return st;
    for (int** p : {&c->cluster_lists, &c->cluster_cnt, &c->cla_lists, &c->cla_cnt}) {
        if (*p) dfree(c, *p);
        *p = nullptr;
    }
    const size_t slots = (size_t)c->cluster_size * c->cluster_per;
    if ((st = dalloc(c, &c->cluster_lists, slots * c->cluster_cap))) return st;
    if ((st = dalloc(c, &c->cluster_cnt, slots))) return st;
    if ((st = dalloc(c, &c->cla_lists, slots * c->cluster_cap))) return st;
    if ((st = dalloc(c, &c->cla_cnt, slots))) return st;
    if (!c->cluster_since && (st = dalloc(c, &c->cluster_since, 1))) return st;
    if (!c->cluster_xref && (st = dalloc(c, &c->cluster_xref, 3 * (size_t)c->n))) return st;
    if (!c->cla_xref && (st = dalloc(c, &c->cla_xref, 3 * (size_t)c->n))) return st;
    return NBG_OK;
}

void prof_begin(nbg_ctx* c)
{
    if (!c->profiling) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, c->stream);
    c->prof_events.push_back(e);
}

void prof_end(nbg_ctx* c)
{
    if (!c->profiling) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, c->stream);
    c->prof_events.push_back(e);
}

static void prof_drain(nbg_ctx* c)
{
    for (size_t k = 0; k + 1 < c->prof_events.size(); k += 2) {
        float ms = 0.f;
        if (cudaEventSynchronize(c->prof_events[k + 1]) == cudaSuccess &&
            cudaEventElapsedTime(&ms, c->prof_events[k], c->prof_events[k + 1]) == cudaSuccess) {
            c->prof_ms += ms;
            c->prof_count++;
        }
        cudaEventDestroy(c->prof_events[k]);
        cudaEventDestroy(c->prof_events[k + 1]);
    }
    c->prof_events.clear();
}

extern "C" int nbg_set_profiling(nbg_ctx* c, int on)
{
    if (!c) return NBG_ERR_ARG;
    NBG_ENTER(c);
    prof_drain(c);
    c->profiling = on != 0;
    c->prof_ms = 0.0;
    c->prof_count = 0;
    return NBG_OK;
}

extern "C" int nbg_force_kernel_time(nbg_ctx* c, double* total_ms, int64_t* launches)
{
    if (!c || !total_ms || !launches) return NBG_ERR_ARG;
    NBG_ENTER(c);
    prof_drain(c);
    *total_ms = c->prof_ms;
    *launches = c->prof_count;
    c->prof_ms = 0.0;
    c->prof_count = 0;
    return NBG_OK;
}

extern "C" int nbg_force_form(nbg_ctx* c, int32_t* lanes, int32_t* fixed_point)
{
    if (!c) return NBG_ERR_ARG;
    if (c->path != PATH_LIST) return fail(c, NBG_ERR_UNSUPPORTED, "the force form applies to the Verlet-list path");
    if (lanes) *lanes = c->list_lpa;
    if (fixed_point) *fixed_point = c->fx_ready ? 1 : 0;
    return NBG_OK;
}

extern "C" int nbg_ensemble_form(nbg_ctx* c, int32_t* lanes, int32_t* threads, int32_t* cells)
{
    if (!c) return NBG_ERR_ARG;
    if (lanes) *lanes = c->ens_ok ? c->ens_lpa : 0;
    if (threads) *threads = c->ens_ok ? c->ens_threads : 0;
    if (cells) *cells = c->ens_ok ? (c->ens_cells == 2 ? 2 : 1) : 0;
    return c->ens_ok ? 1 : 0;
}

extern "C" int nbg_cluster_launch_floor(nbg_ctx* c, double* us_single, double* us_per_launch)
{
    if (!c) return NBG_ERR_ARG;
    NBG_ENTER(c);
    return cluster_launch_floor(c, us_single, us_per_launch);
}

extern "C" int nbg_cluster_shape(nbg_ctx* c, int32_t* ctas, int32_t* lanes)
{
    if (!c) return NBG_ERR_ARG;
    if (ctas) *ctas = c->cluster_ok ? c->cluster_size : 0;
    if (lanes) *lanes = c->cluster_ok ? c->cluster_lpa : 0;
    return c->cluster_ok ? 1 : 0;
}

static void release(nbg_ctx* c)
{
    prof_drain(c);
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
    if (c->accel_graph) cudaGraphExecDestroy(c->accel_graph);
    c->accel_graph = nullptr;
    if (c->hst) cudaFreeHost(c->hst);
    c->hst = nullptr;
    if (c->hw) cudaFreeHost(c->hw);
    c->hw = c->hw_d = nullptr;
    if (c->pend_ev) cudaEventDestroy(c->pend_ev);
    c->pend_ev = nullptr;
    if (c->frames) cudaFree(c->frames);
    c->frames = nullptr;
    c->frames_cap = 0;
    for (void* p : c->allocs) cudaFree(p);
    c->allocs.clear();
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    c->own_stream = nullptr;
}

extern "C" int nbg_create_batch(const nbg_system_desc* descs, int32_t n_replicas, int device, nbg_ctx** out)
{
    NBG_RANGE("nbg_create_batch");
    if (!out) return NBG_ERR_ARG;
    *out = nullptr;
    if (!descs || n_replicas < 1) return NBG_ERR_ARG;
    std::string why;
    for (int r = 0; r < n_replicas; ++r) {
        int v = validate(&descs[r], why);
        if (v) {
            fprintf(stderr, "nbg_create: replica %d: %s\n", r, why.c_str());
            return v;
        }
    }
    const nbg_system_desc* d0 = &descs[0];
    for (int r = 1; r < n_replicas; ++r) {
        const nbg_system_desc* d = &descs[r];
        if (d->kind != d0->kind || d->potentials != d0->potentials || d->thermostat != d0->thermostat ||
            d->bc != d0->bc || d->lj_cutoff != d0->lj_cutoff || d->el_cutoff != d0->el_cutoff ||
            d->lj_sigma != d0->lj_sigma || d->lj_epsilon != d0->lj_epsilon || d->el_k != d0->el_k ||
            d->skin != d0->skin || d->kb != d0->kb) {
            fprintf(stderr, "nbg_create_batch: replica %d differs in kind/potentials/parameters\n", r);
            return NBG_ERR_ARG;
        }
    }
    if (n_replicas > 1 && d0->thermostat == NBG_THERMO_NOSEHOOVER) {
        fprintf(stderr, "nbg_create_batch: Nose-Hoover batches are not supported\n");
        return NBG_ERR_UNSUPPORTED;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        fprintf(stderr, "nbg_create: CUDA device %d not available\n", device);
        return NBG_ERR_CUDA;
    }
    if (cudaSetDevice(device) != cudaSuccess) return NBG_ERR_CUDA;
    nbg_ctx* c = new nbg_ctx();
    c->device = device;
    if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return NBG_ERR_CUDA;
    }
    c->stream = c->own_stream;
    int st = build_context(c, descs, n_replicas);
    if (st != NBG_OK) {
        fprintf(stderr, "nbg_create: %s\n", c->err.c_str());
        release(c);
        delete c;
        return st;
    }
    *out = c;
    return NBG_OK;
}

extern "C" int nbg_create(const nbg_system_desc* desc, int device, nbg_ctx** out)
{
    return nbg_create_batch(desc, 1, device, out);
}

extern "C" void nbg_destroy(nbg_ctx* c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->pending) cudaStreamSynchronize(c->stream);  // queued steps end before the buffers go
    if (c->stream) cudaStreamSynchronize(c->stream);
    release(c);
    delete c;
}

extern "C" int nbg_set_stream(nbg_ctx* c, void* s)
{
    if (!c) return NBG_ERR_ARG;
    NBG_ENTER(c);  // deferred steps on the previous stream settle first
    c->stream = s ? (cudaStream_t)s : c->own_stream;
    return NBG_OK;
}

// ---------------------------------------------------------------------
// forces and status
// ---------------------------------------------------------------------
static int read_status(nbg_ctx* c, unsigned* st)
{
    CK(cudaMemcpyAsync(st, c->d.status, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream), "status read");
    CK(cudaStreamSynchronize(c->stream), "stream sync");
    return NBG_OK;
}

static int clear_status(nbg_ctx* c)
{
    CK(cudaMemsetAsync(c->d.status, 0, sizeof(unsigned), c->stream), "status clear");
    return NBG_OK;
}

// The pinned, mapped status word and the event that follows a deferred chunk
// (allocated once per context).
static int ensure_hw(nbg_ctx* c)
{
    if (c->hw) return NBG_OK;
    unsigned* h = nullptr;
    if (cudaHostAlloc((void**)&h, 64, cudaHostAllocMapped) != cudaSuccess) {
        cudaGetLastError();
        return fail(c, NBG_ERR_NOMEM, "pinned status word: cudaHostAlloc failed");
    }
    *h = 0u;
    c->hw = h;
    CK(cudaHostGetDevicePointer((void**)&c->hw_d, h, 0), "status word device pointer");
    CK(cudaEventCreateWithFlags(&c->pend_ev, cudaEventDisableTiming), "pending event");
    return NBG_OK;
}

static int status_error(nbg_ctx* c, unsigned st)
{
    if (st & ST_INDEX) return fail(c, NBG_ERR_INDEX, "a neighbour or cell index out of range (debug build check)");
    if (st & ST_NONFINITE) return fail(c, NBG_ERR_NONFINITE, "non-finite acceleration (NaN/Inf state or coincident bodies)");
    if (st & ST_RANGE) return fail(c, NBG_ERR_RANGE, "minimum-image loop exceeded its iteration cap");
    if (st & ST_TIMEOUT) return fail(c, NBG_ERR_TIMEOUT, "a device-side wait for data from other blocks ran out");
    if (st & (ST_CELL_OVERFLOW | ST_NBR_OVERFLOW | ST_SHORT_OVERFLOW))
        return fail(c, NBG_ERR_CAPACITY, "list capacity exceeded");
    return NBG_OK;
}

// Potential accelerations of state s into s.a_new (no thermostat term).
// pos: time index of the positions in s (its parity picks the rebuild flag).
static int forces(nbg_ctx* c, const StateView& s, bool force_build, StepRef pos)
{
    NBG_RANGE("forces");
    int st = NBG_OK;
    if (c->path == PATH_GRAVITY) {
        st = launch_gravity(c, s);
    } else if (c->path == PATH_LIST) {
        if ((st = launch_list_build(c, s, force_build, pos))) return st;
#ifdef NBG_DEBUG
        if (c->plant_index) {
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            CK(cudaStreamIsCapturing(c->stream, &cs), "capture query");
            if (cs == cudaStreamCaptureStatusNone) {
                if ((st = launch_plant_index(c, c->plant_index))) return st;
                c->plant_index = 0;
            }
        }
#endif
        st = launch_force_list(c, s);
    } else {
        st = launch_allpairs(c, s);
    }
    if (st) return st;
    if (c->d.kind == NBG_SYSTEM_WATER) st = launch_bonded(c, s);
    return st;
}

// grow the list capacities after an overflow
static int grow_lists(nbg_ctx* c, unsigned st)
{
    int cell_cap = c->d.cell_cap, nbr_cap = c->d.nbr_cap;
    if (st & ST_CELL_OVERFLOW) cell_cap *= 2;
    if (st & ST_NBR_OVERFLOW) nbr_cap = nbr_cap + nbr_cap / 2 + 32;
    // the per-cell sort stages a cell in 48 KB of shared memory
    if (cell_cap > 12288)
        return fail(c, NBG_ERR_CAPACITY, "more than 12288 atoms in one cell: the configuration has collapsed");
    if (c->graph) {  // the captured kernels hold the old list pointers
        cudaGraphExecDestroy(c->graph);
        c->graph = nullptr;
    }
    int rc = alloc_lists(c, cell_cap, nbr_cap);  // (drops the right-hand-side graph too)
    if (rc) return rc;
    return plan_cluster(c);  // the lists' shared-memory share grew
}

// Evaluate forces on a one-off state (scratch view), retrying on overflow.
static int forces_once(nbg_ctx* c, const StateView& s)
{
    for (int attempt = 0; attempt < 6; ++attempt) {
        int st;
        if ((st = clear_status(c))) return st;
        if ((st = launch_pack(c, s))) return st;
        if ((st = forces(c, s, true, StepRef{0, nullptr}))) return st;
        unsigned w = 0;
        if ((st = read_status(c, &w))) return st;
        if (w & ST_FATAL) return status_error(c, w);
        if (w & (ST_CELL_OVERFLOW | ST_NBR_OVERFLOW)) {
            if ((st = grow_lists(c, w))) return st;
            continue;
        }
        return status_error(c, w);
    }
    return fail(c, NBG_ERR_CAPACITY, "list capacity could not be grown enough");
}

static size_t state_bytes(const nbg_ctx* c) { return sizeof(double) * 3 * (size_t)c->cols; }

// The scratch view shares the split positions and the lists with the
// resident state: the next resident step rebuilds the lists (every step
// repacks the positions anyway).
static void resident_dirty(nbg_ctx* c)
{
    c->steps_since_build = -1;
    c->respa_valid = false;
    c->cluster_lists_valid = false;
    c->ens_lists_valid = false;
}

// The list path's right-hand side as one captured graph of kernels only:
// an import node reads u (and v) from the pinned staging (mapped host
// memory, read by the GPU over the CPU-GPU link), stores and packs them,
// checks the displacement against the last build and clears the status;
// the list kernels rebuild only when flagged; the force kernels and the
// thermostat term; an export node writes dv (and the Nose-Hoover rate) and
// the status word back into the staging and advances the call counter
// whose parity picks the rebuild flags.
static int ensure_staging(nbg_ctx* c, double** dev)
{
    if (!c->hst) {
        cudaError_t e = cudaHostAlloc((void**)&c->hst, 3 * state_bytes(c) + 64, cudaHostAllocMapped);
        if (e != cudaSuccess) {
            cudaGetLastError();
            c->hst = nullptr;
            return fail(c, NBG_ERR_NOMEM, "pinned staging of the right-hand side: cudaHostAlloc failed");
        }
    }
    CK(cudaHostGetDevicePointer((void**)dev, c->hst, 0), "staging device pointer");
    return NBG_OK;
}

static int accel_graph_capture(nbg_ctx* c, bool v_read)
{
    double* dst = nullptr;
    int st;
    if ((st = ensure_staging(c, &dst))) return st;
    if (!c->accel_step && (st = dalloc(c, &c->accel_step, 1))) return st;
    const int64_t launches0 = c->launches;
    const StepRef pos{0, c->accel_step};
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "accel capture begin");
    st = launch_accel_import(c, c->ev, dst, dst + 3 * c->cols, v_read, pos);
    if (st == NBG_OK) st = forces(c, c->ev, false, pos);
    if (st == NBG_OK) st = launch_rhs_thermostat(c, c->ev);
    if (st == NBG_OK)
        st = launch_accel_export(c, c->ev, dst + 6 * c->cols, dst + 3 * c->cols,
                                 reinterpret_cast<unsigned*>(dst + 9 * c->cols), c->accel_step);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    c->accel_graph_launches = c->launches - launches0;
    c->launches = launches0;
    c->accel_lists_valid = false;  // nothing ran yet: the first replay builds
    if (st != NBG_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "accel capture");
    e = cudaGraphInstantiate(&c->accel_graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        c->accel_graph = nullptr;
        return cuda_fail(c, e, "accel graph instantiate");
    }
    return NBG_OK;
}

// The device address of a host buffer of `bytes` that the device can read
// and write in place (page-locked, mapped, one piece from its first to its
// last byte), else null.
static void* mapped_address(const void* p, size_t bytes)
{
    cudaPointerAttributes a0{}, a1{};
    if (cudaPointerGetAttributes(&a0, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a0.type != cudaMemoryTypeHost || !a0.devicePointer) return nullptr;
    if (cudaPointerGetAttributes(&a1, static_cast<const char*>(p) + bytes - 1) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a1.type != cudaMemoryTypeHost ||
        static_cast<char*>(a1.devicePointer) - static_cast<char*>(a0.devicePointer) != (ptrdiff_t)(bytes - 1))
        return nullptr;
    return a0.devicePointer;
}

// nbg_accel of a small system (the cluster path): one launch reads u and
// writes dv in place when they are page-locked host buffers, else through
// the pinned staging; the status word comes back through the mapped word.
// Returns 1 when the cluster path no longer applies (lists grew past it).
static int accel_cluster(nbg_ctx* c, double* dv, const double* u)
{
    int st;
    double* stage = nullptr;
    if ((st = ensure_hw(c))) return st;
    const size_t sb = sizeof(double) * 3 * (size_t)c->n;
    const double* ud = static_cast<const double*>(mapped_address(u, sb));
    double* dvd = static_cast<double*>(mapped_address(dv, sb));
    if ((!ud || !dvd) && (st = ensure_staging(c, &stage))) return st;
    if (!ud) {
        memcpy(c->hst, u, sb);
        ud = stage;
    }
    double* out = dvd ? dvd : stage + 6 * c->cols;
    for (int attempt = 0; attempt < 6; ++attempt) {
        *(volatile unsigned*)c->hw = 0u;
        if ((st = launch_cluster_accel(c, ud, out, c->hw_d))) return st;
        CK(cudaStreamSynchronize(c->stream), "accel sync");
        const unsigned w = *(volatile unsigned*)c->hw;
        c->cla_valid = w == 0u;
        if (w & (ST_CELL_OVERFLOW | ST_NBR_OVERFLOW)) {
            if ((st = grow_lists(c, w))) return st;
            if (!c->cluster_ok) return 1;
            continue;
        }
        if (w) return status_error(c, w);
        if (!dvd) memcpy(dv, c->hst + 6 * c->cols, sb);
        return NBG_OK;
    }
    return fail(c, NBG_ERR_CAPACITY, "list capacity could not be grown enough");
}

extern "C" int nbg_accel(nbg_ctx* c, double* dv, double* v, const double* u, double t)
{
    NBG_RANGE("nbg_accel");
    (void)t;
    if (!c || !dv || !v || !u) return NBG_ERR_ARG;
    NBG_ENTER(c);
    // only the Berendsen and Nose-Hoover terms of the right-hand side read v
    const bool v_read = c->d.therm == NBG_THERMO_BERENDSEN || c->d.therm == NBG_THERMO_NOSEHOOVER;
    if (c->path == PATH_LIST && c->cluster_ok) {
        // (no thermostat term: the cluster path serves plain systems only)
        const int st = accel_cluster(c, dv, u);
        if (st != 1) return st;
    }
    if (c->path == PATH_LIST && c->use_graphs && !c->profiling) {
        resident_dirty(c);
        c->T_valid = false;
        for (int attempt = 0; attempt < 6; ++attempt) {
            int st;
            if (!c->accel_graph && (st = accel_graph_capture(c, v_read))) return st;
            const size_t sb = state_bytes(c);
            memcpy(c->hst, u, sb);
            if (v_read) memcpy(c->hst + 3 * c->cols, v, sb);
            if (!c->accel_lists_valid)  // lists of other positions: every replica rebuilds
                CK(cudaMemsetAsync(c->d.rebuild_flag, 0xff, 2 * sizeof(int) * (size_t)c->nrep, c->stream), "flags");
            CK(cudaGraphLaunch(c->accel_graph, c->stream), "accel graph launch");
            c->launches += c->accel_graph_launches;
            CK(cudaStreamSynchronize(c->stream), "accel sync");
            const unsigned w = *reinterpret_cast<const unsigned*>(c->hst + 9 * c->cols);
            if (w & ST_FATAL) return status_error(c, w);
            if (w & (ST_CELL_OVERFLOW | ST_NBR_OVERFLOW)) {
                if ((st = grow_lists(c, w))) return st;  // (drops the graph: captured again above)
                continue;
            }
            memcpy(dv, c->hst + 6 * c->cols, sb);
            if (c->d.therm == NBG_THERMO_NOSEHOOVER) v[3 * c->n] = c->hst[3 * c->cols + 3 * c->n];
            c->accel_lists_valid = true;
            return status_error(c, w);
        }
        return fail(c, NBG_ERR_CAPACITY, "list capacity could not be grown enough");
    }
    CK(cudaMemcpyAsync(c->ev.x, u, state_bytes(c), cudaMemcpyHostToDevice, c->stream), "u upload");
    if (v_read) CK(cudaMemcpyAsync(c->ev.v, v, state_bytes(c), cudaMemcpyHostToDevice, c->stream), "v upload");
    resident_dirty(c);
    c->T_valid = false;  // the RHS reduces T of its own velocities into red_T
    // the whole evaluation, the download and the status word in one stream
    // pass with one synchronisation; a list overflow grows the lists and
    // evaluates again
    for (int attempt = 0; attempt < 6; ++attempt) {
        int st;
        if ((st = clear_status(c))) return st;
        CK(cudaMemsetAsync(c->ev.a_new, 0, state_bytes(c), c->stream), "dv clear");
        // the sorted gravity path packs its own (permuted) split positions
        if (!(c->path == PATH_GRAVITY && c->grav_sort) && (st = launch_pack(c, c->ev))) return st;
        if ((st = forces(c, c->ev, true, StepRef{0, nullptr}))) return st;
        if ((st = launch_rhs_thermostat(c, c->ev))) return st;
        CK(cudaMemcpyAsync(dv, c->ev.a_new, state_bytes(c), cudaMemcpyDeviceToHost, c->stream), "dv download");
        if (c->d.therm == NBG_THERMO_NOSEHOOVER)
            CK(cudaMemcpyAsync(v + 3 * c->n, c->ev.v + 3 * c->n, sizeof(double), cudaMemcpyDeviceToHost, c->stream),
               "v download");
        unsigned w = 0;
        if ((st = read_status(c, &w))) return st;
        if (w & ST_FATAL) return status_error(c, w);
        if (w & (ST_CELL_OVERFLOW | ST_NBR_OVERFLOW)) {
            if ((st = grow_lists(c, w))) return st;
            continue;
        }
        return status_error(c, w);
    }
    return fail(c, NBG_ERR_CAPACITY, "list capacity could not be grown enough");
}

extern "C" int nbg_set_state(nbg_ctx* c, const double* u, const double* v)
{
    NBG_RANGE("nbg_set_state");
    if (!c || !u || !v) return NBG_ERR_ARG;
    NBG_ENTER(c);
    CK(cudaMemcpyAsync(c->st.x, u, state_bytes(c), cudaMemcpyHostToDevice, c->stream), "u upload");
    CK(cudaMemcpyAsync(c->st.v, v, state_bytes(c), cudaMemcpyHostToDevice, c->stream), "v upload");
    c->state_valid = true;
    c->accel_valid = false;
    c->respa_valid = false;
    c->T_valid = false;
    c->steps_since_build = -1;
    c->cluster_lists_valid = false;
    c->ens_lists_valid = false;
    // the gravity sort schedule restarts too: runs from the same state give
    // the same bits
    c->grav_evals = 0;
    c->grav_perm_valid = false;
    return NBG_OK;
}

extern "C" int nbg_get_state(nbg_ctx* c, double* u, double* v)
{
    NBG_RANGE("nbg_get_state");
    if (!c || (!u && !v)) return NBG_ERR_ARG;
    NBG_ENTER(c);
    if (u) CK(cudaMemcpyAsync(u, c->st.x, state_bytes(c), cudaMemcpyDeviceToHost, c->stream), "u download");
    if (v) CK(cudaMemcpyAsync(v, c->st.v, state_bytes(c), cudaMemcpyDeviceToHost, c->stream), "v download");
    CK(cudaStreamSynchronize(c->stream), "state sync");
    return NBG_OK;
}

extern "C" int nbg_get_step(nbg_ctx* c, int64_t* step)
{
    if (!c || !step) return NBG_ERR_ARG;
    *step = c->step;
    return NBG_OK;
}

extern "C" int nbg_set_step(nbg_ctx* c, int64_t step)
{
    if (!c) return NBG_ERR_ARG;
    NBG_ENTER(c);
    if (step < 0) return fail(c, NBG_ERR_ARG, "the step counter must be >= 0");
    c->step = step;
    return NBG_OK;
}

extern "C" int nbg_compute_forces(nbg_ctx* c)
{
    NBG_RANGE("nbg_compute_forces");
    if (!c) return NBG_ERR_ARG;
    if (!c->state_valid) return fail(c, NBG_ERR_ARG, "no resident state (call nbg_set_state)");
    NBG_ENTER(c);
    int st;
    if ((st = launch_pack(c, c->st))) return st;
    if ((st = forces(c, c->st, c->steps_since_build < 0, StepRef{c->step, nullptr}))) return st;
    if (c->steps_since_build < 0) c->steps_since_build = 0;
    return NBG_OK;
}

extern "C" int nbg_get_accel(nbg_ctx* c, double* dv)
{
    NBG_RANGE("nbg_get_accel");
    if (!c || !dv) return NBG_ERR_ARG;
    NBG_ENTER(c);
    CK(cudaMemcpyAsync(dv, c->st.a_new, state_bytes(c), cudaMemcpyDeviceToHost, c->stream), "a download");
    CK(cudaStreamSynchronize(c->stream), "accel sync");
    unsigned w = 0;
    int st = read_status(c, &w);
    if (st) return st;
    return status_error(c, w);
}

// ---------------------------------------------------------------------
// the step loop
// ---------------------------------------------------------------------
// The step loop's backup buffer (allocated once per context).
static int ensure_backup(nbg_ctx* c)
{
    return c->bk ? NBG_OK : dalloc(c, &c->bk, 12 * (size_t)c->cols);
}

// x, v, a_old of the resident state to the backup (one copy), or the n atoms'
// rows of each back (one strided copy: the cluster loop writes the backup of
// its atoms itself, not the padding)
static int backup_state(nbg_ctx* c, bool restore)
{
    const size_t seg = 3 * sizeof(double) * (size_t)c->cols;
    if (restore) {
        CK(cudaMemcpy2DAsync(c->st.x, seg, c->bk, seg, 3 * sizeof(double) * (size_t)c->n, 3,
                             cudaMemcpyDeviceToDevice, c->stream),
           "restore");
    } else {
        CK(cudaMemcpyAsync(c->bk, c->st.x, 3 * seg, cudaMemcpyDeviceToDevice, c->stream), "backup");
    }
    return NBG_OK;
}

// The status of the chunk just launched (synchronises the stream).
static int chunk_status(nbg_ctx* c, unsigned* w)
{
    if (!c->chunk_hw) return read_status(c, w);
    CK(cudaStreamSynchronize(c->stream), "stream sync");
    *w = *(volatile unsigned*)c->hw;
    return NBG_OK;
}

// EM is the reference's Langevin integrator; BAOAB (flag) and velocity
// Verlet share the kick-drift structure.
static bool is_em(const nbg_ctx* c) { return c->d.therm == NBG_THERMO_LANGEVIN && !c->baoab; }

// a_old = f(v, u) at the current resident state (SciML computes the first
// acceleration before the first step; with Nose-Hoover this also writes the
// rate into v, as the reference's RHS does).
static int init_accel(nbg_ctx* c)
{
    int st;
    if ((st = launch_pack(c, c->st))) return st;
    if ((st = forces(c, c->st, true, StepRef{c->step, nullptr}))) return st;
    c->steps_since_build = 0;
    if (!is_em(c)) {
        if ((st = launch_rhs_thermostat(c, c->st))) return st;
        CK(cudaMemcpyAsync(c->st.a_old, c->st.a_new, state_bytes(c), cudaMemcpyDeviceToDevice, c->stream), "a init");
        c->T_valid = true;
    }
    c->accel_valid = true;
    return NBG_OK;
}

// Is the host-forced list rebuild due at this step? (VV: positions advance
// before the forces; EM: the forces use the current positions.)
static bool rebuild_due(const nbg_ctx* c, bool vv)
{
    if (c->path != PATH_LIST) return false;
    int re = c->desc.rebuild_every;
    if (c->steps_since_build < 0) return true;
    return re > 0 && (vv ? c->steps_since_build + 1 : c->steps_since_build) >= re;
}

// One step. sr: the step index (absolute, or an offset from the device step
// counter inside a captured graph).
static int step_vv(nbg_ctx* c, double dt, StepRef sr)
{
    int st;
    const StateView& s = c->st;
    StepRef pos{sr.off + 1, sr.base};
    if ((st = launch_drift(c, s, dt, pos))) return st;
    bool force = rebuild_due(c, true);
    if ((st = forces(c, s, force, pos))) return st;
    c->steps_since_build = force ? 0 : c->steps_since_build + 1;
    const bool thermo_T = c->d.therm == NBG_THERMO_BERENDSEN || c->d.therm == NBG_THERMO_NOSEHOOVER;
    // single systems fold the next step's T into the kick; batches reduce per replica
    const bool fused_T = thermo_T && c->nrep == 1;
    if (thermo_T && !(fused_T && c->T_valid))
        if ((st = launch_temperature(c, s.v))) return st;
    if ((st = launch_kick(c, s, dt, fused_T))) return st;
    c->T_valid = fused_T;
    if (c->d.therm == NBG_THERMO_ANDERSEN)
        if ((st = launch_andersen(c, s, dt, sr))) return st;
    return NBG_OK;
}

static int step_baoab(nbg_ctx* c, double dt, StepRef sr)
{
    int st;
    const StateView& s = c->st;
    StepRef pos{sr.off + 1, sr.base};
    if ((st = launch_baoab_drift(c, s, dt, sr))) return st;
    bool force = rebuild_due(c, true);
    if ((st = forces(c, s, force, pos))) return st;
    c->steps_since_build = force ? 0 : c->steps_since_build + 1;
    return launch_baoab_kick(c, s, dt);
}

// A BAOAB step inside a captured run of steps: the first drifts alone, the
// others fold the previous step's kick into their drift, and the last kicks.
static int step_baoab_fused(nbg_ctx* c, double dt, StepRef sr, bool first, bool last)
{
    int st;
    const StateView& s = c->st;
    StepRef pos{sr.off + 1, sr.base};
    if ((st = first ? launch_baoab_drift(c, s, dt, sr) : launch_baoab_kick_drift(c, s, dt, sr))) return st;
    bool force = rebuild_due(c, true);
    if ((st = forces(c, s, force, pos))) return st;
    c->steps_since_build = force ? 0 : c->steps_since_build + 1;
    return last ? launch_baoab_kick(c, s, dt) : NBG_OK;
}

static int step_em(nbg_ctx* c, double dt, StepRef sr)
{
    int st;
    const StateView& s = c->st;
    bool force = rebuild_due(c, false);
    if ((st = forces(c, s, force, sr))) return st;
    c->steps_since_build = force ? 1 : c->steps_since_build + 1;
    if ((st = launch_em(c, s, dt, sr))) return st;
    return NBG_OK;
}

static int step_any(nbg_ctx* c, double dt, StepRef sr)
{
    int st = is_em(c) ? step_em(c, dt, sr) : c->baoab ? step_baoab(c, dt, sr) : step_vv(c, dt, sr);
    if (st == NBG_OK && c->sink_on) st = launch_save_frame(c, c->st, sr);
    return st;
}

static int step_direct(nbg_ctx* c, double dt)
{
    int st = step_any(c, dt, StepRef{c->step, nullptr});
    if (st) return st;
    c->step++;
    return NBG_OK;
}

// Steps per captured graph: one rebuild period (so the host-forced rebuilds
// fall on the same graph steps every replay), at least 8.
static int64_t graph_period(const nbg_ctx* c)
{
    int64_t g = c->path == PATH_LIST && c->desc.rebuild_every > 0 ? c->desc.rebuild_every : 1;
    while (g < 8) g *= 2;
    return g;
}

// A replay starts where the host pattern of forced rebuilds matches the
// capture: right after a rebuild period (or with a rebuild pending).
static bool graph_aligned(const nbg_ctx* c)
{
    if (c->path != PATH_LIST) return true;
    // displacement-only rebuilds: capture once the first (forced) build is done
    if (c->desc.rebuild_every <= 0) return c->steps_since_build >= 0;
    bool vv = !is_em(c);
    int re = c->desc.rebuild_every;
    int64_t s = c->steps_since_build;
    return vv ? (s < 0 || s + 1 >= re) : (s < 0 || s >= re);
}

// Capture graph_period() steps on the context stream (kernels read the step
// counter from device memory, the last node advances it) and instantiate.
static int capture_graph(nbg_ctx* c, double dt)
{
    if (c->graph) {
        cudaGraphExecDestroy(c->graph);
        c->graph = nullptr;
    }
    const int64_t G = graph_period(c);
    if ((c->d.therm == NBG_THERMO_BERENDSEN || c->d.therm == NBG_THERMO_NOSEHOOVER) && c->nrep == 1 && !c->T_valid) {
        int st0 = launch_temperature(c, c->st.v);
        if (st0) return st0;
        c->T_valid = true;
    }
    const int64_t launches0 = c->launches;
    const int64_t ssb0 = c->steps_since_build;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "graph capture begin");
    int st = NBG_OK;
    // (BAOAB without frames: each kick folded into the next step's drift)
    const bool fuse = c->baoab && !is_em(c) && !c->sink_on;
    for (int64_t k = 0; k < G && st == NBG_OK; ++k)
        st = fuse ? step_baoab_fused(c, dt, StepRef{k, c->d.step_dev}, k == 0, k == G - 1)
                  : step_any(c, dt, StepRef{k, c->d.step_dev});
    if (st == NBG_OK) st = launch_step_advance(c, G);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    c->steps_since_build = ssb0;  // capture only recorded the steps
    c->T_valid = (c->d.therm == NBG_THERMO_BERENDSEN || c->d.therm == NBG_THERMO_NOSEHOOVER) && c->nrep == 1;
    if (st != NBG_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "graph capture");
    e = cudaGraphInstantiate(&c->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        c->graph = nullptr;
        return cuda_fail(c, e, "graph instantiate");
    }
    c->graph_steps = G;
    c->graph_sink = c->sink_on;
    c->graph_launches = c->launches - launches0;
    c->launches = launches0;
    c->graph_dt = dt;
    return NBG_OK;
}

// Replay the step graph once: graph_period() steps.
static int replay_graph(nbg_ctx* c)
{
    CK(cudaGraphLaunch(c->graph, c->stream), "graph launch");
    c->launches += c->graph_launches;
    c->step += c->graph_steps;
    // the forced-rebuild pattern repeats: after a period the host state is as at capture
    bool vv = !is_em(c);
    if (c->path == PATH_LIST && c->desc.rebuild_every > 0) {
        int64_t re = c->desc.rebuild_every;
        c->steps_since_build = vv ? re - 1 : re;
        (void)re;
    }
    return NBG_OK;
}

// device bytes of trajectory frames (positions and velocities) nbg_run keeps
// before copying them out
#define RUN_FRAME_BYTES ((size_t)1 << 30)

static int advance_impl(nbg_ctx* c, double dt, int64_t nsteps, bool defer = false);

// Read the status word of a deferred nbg_advance chunk. After a list
// overflow the chunk is undone (backup), the lists grow, and it runs again
// (synchronously); a non-finite, range or timeout status is returned here.
static int settle(nbg_ctx* c)
{
    if (!c->pending) return NBG_OK;
    c->pending = false;
    // the chunk alone (its status word was set or copied before the event)
    CK(cudaEventSynchronize(c->pend_ev), "pending chunk");
    const unsigned w = *(volatile unsigned*)c->hw;
    int st;
    if (w & ST_TIMEOUT) {
        if ((st = backup_state(c, true))) return st;  // the chunk ended early: back to its start
        c->step = c->pend_step0;
        c->steps_since_build = -1;
        c->cluster_lists_valid = false;
        c->ens_lists_valid = false;
        c->T_valid = false;
        return status_error(c, ST_TIMEOUT);
    }
    if (w & (ST_NONFINITE | ST_RANGE | ST_INDEX)) return status_error(c, w);
    if (w & (ST_CELL_OVERFLOW | ST_NBR_OVERFLOW)) {
        if ((st = grow_lists(c, w))) return st;
        if ((st = backup_state(c, true))) return st;
        c->step = c->pend_step0;
        c->steps_since_build = -1;
        c->cluster_lists_valid = false;
        c->ens_lists_valid = false;
        c->T_valid = false;
        if ((st = clear_status(c))) return st;
        if ((st = launch_pack(c, c->st))) return st;
        return advance_impl(c, c->pend_dt, c->pend_steps, false);
    }
    return status_error(c, w);
}

// defer: leave the status of the last chunk unread (no host synchronisation);
// the next call on the context settles it.
static int advance_impl(nbg_ctx* c, double dt, int64_t nsteps, bool defer)
{
    if (!c->state_valid) return fail(c, NBG_ERR_ARG, "no resident state (call nbg_set_state)");
    if (!(dt > 0.0) || nsteps < 0) return fail(c, NBG_ERR_ARG, "dt must be > 0 and nsteps >= 0");
    int st;
    c->respa_valid = false;  // a_old becomes the velocity-Verlet acceleration
    c->accel_lists_valid = false;  // the steps rebuild the lists for the resident positions
    if (c->baoab && c->baoab_dt != dt) {
        // per-replica BAOAB coefficients for this dt (host FP64, uploaded before any capture)
        for (int r = 0; r < c->nrep; ++r) {
            RepDev& R = c->reps_h[r];
            R.bc1 = std::exp(-R.tparam * dt);
            R.bsd = std::sqrt(1.0 - R.bc1 * R.bc1) * std::sqrt(c->d.kb * R.T0);
        }
        CK(cudaMemcpyAsync(const_cast<RepDev*>(c->d.reps), c->reps_h.data(), sizeof(RepDev) * c->nrep,
                           cudaMemcpyHostToDevice, c->stream), "replica upload");
        CK(cudaStreamSynchronize(c->stream), "replica sync");
        c->baoab_dt = dt;
        if (c->graph) {
            cudaGraphExecDestroy(c->graph);
            c->graph = nullptr;
        }
    }
    const bool em = is_em(c);
    const bool can_overflow = c->path == PATH_LIST;
    if (can_overflow && ((st = ensure_backup(c)) || (st = ensure_hw(c)))) return st;
    // chunks run as one launch (cluster or ensemble loop) on a state whose
    // acceleration is known report to the host word: the device word is
    // neither cleared nor read in this call
    const bool hw_ok = can_overflow && !em && c->accel_valid && (c->cluster_ok || c->ens_ok);
    if (!hw_ok && (st = clear_status(c))) return st;
    if (!em && !c->accel_valid) {
        if ((st = init_accel(c))) return st;
    } else if (em) {
        if ((st = launch_pack(c, c->st))) return st;
    }
    const int64_t chunk = can_overflow ? 512 : nsteps;
    // graphs pay off for short steps; events around kernels (profiling) stay direct
    const bool graphs = c->use_graphs && !c->profiling && nsteps >= 2 * graph_period(c);
    int64_t done = 0;
    int retries = 0;
    while (done < nsteps) {
        int64_t k = std::min<int64_t>(chunk > 0 ? chunk : nsteps, nsteps - done);
        const int64_t step0 = c->step;
        // (a retry below clears the device word, so a chunk that falls back
        // from the one-launch loops to graphs reads a clean word)
        c->chunk_hw = hw_ok && (c->cluster_ok || c->ens_ok);
        if (c->chunk_hw) *(volatile unsigned*)c->hw = 0u;  // no launch that sets it is in flight
        // the cluster loop writes the backup of its atoms itself
        if (can_overflow && !(c->chunk_hw && c->cluster_ok) && (st = backup_state(c, false))) return st;
        int64_t s = 0;
        bool counter_set = false;
        while (s < k) {
            if (c->ens_ok && !is_em(c)) {
                // every replica's steps of the chunk in one launch (a CTA per
                // replica; its lists stay with it between launches)
                if ((st = launch_ensemble(c, c->st, dt, k - s, c->step, c->chunk_hw ? c->hw_d : c->d.status))) break;
                c->ens_lists_valid = true;
                c->step += k - s;
                c->steps_since_build = -1;
                s = k;
                continue;
            }
            if (c->cluster_ok) {
                // the whole chunk in one persistent cluster launch (its lists
                // live in shared memory: the global ones are rebuilt later)
                if ((st = launch_cluster_vv(c, c->st, dt, k - s, c->desc.rebuild_every, c->step,
                                             c->chunk_hw ? c->hw_d : c->d.status)))
                    break;
                c->cluster_lists_valid = true;
                c->step += k - s;
                c->steps_since_build = -1;
                s = k;
                continue;
            }
            c->cluster_lists_valid = false;
            c->ens_lists_valid = false;  // the graph or direct steps below move the state
            if (graphs && graph_aligned(c) && k - s >= graph_period(c)) {
                if (!c->graph || c->graph_dt != dt || c->graph_sink != c->sink_on) {
                    if ((st = capture_graph(c, dt))) break;
                }
                if (!counter_set) {
                    if ((st = launch_set_step(c, c->step))) break;
                    counter_set = true;
                }
                if ((st = replay_graph(c))) break;
                s += c->graph_steps;
            } else {
                if ((st = step_direct(c, dt))) break;
                counter_set = false;
                ++s;
            }
        }
        if (st) return st;
        if (defer && done + k == nsteps && can_overflow) {
            // the last chunk's status is read by the next call (settle)
            if (!c->chunk_hw) {
                CK(cudaMemcpyAsync(c->hw, c->d.status, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream),
                   "status copy");
            }
            CK(cudaEventRecord(c->pend_ev, c->stream), "pending event");
            c->pending = true;
            c->pend_dt = dt;
            c->pend_steps = k;
            c->pend_step0 = step0;
            return NBG_OK;
        }
        unsigned w = 0;
        if ((st = chunk_status(c, &w))) return st;
        if ((w & ST_TIMEOUT) && can_overflow) {
            // a launch that gave up waiting ended early: the state goes back
            // to the chunk's start, and the error is returned
            if ((st = backup_state(c, true))) return st;
            c->step = step0;
            c->steps_since_build = -1;
            c->cluster_lists_valid = false;
            c->ens_lists_valid = false;
            c->T_valid = false;
            return status_error(c, ST_TIMEOUT);  // (whatever else the abandoned steps flagged)
        }
        if (w & ST_FATAL) return status_error(c, w);
        if (w & (ST_CELL_OVERFLOW | ST_NBR_OVERFLOW)) {
            if (++retries > 6) return fail(c, NBG_ERR_CAPACITY, "list capacity could not be grown enough");
            if ((st = grow_lists(c, w))) return st;
            if ((st = backup_state(c, true))) return st;
            c->step = step0;
            c->steps_since_build = -1;
            c->cluster_lists_valid = false;
            c->ens_lists_valid = false;
            c->T_valid = false;
            if ((st = clear_status(c))) return st;
            if ((st = launch_pack(c, c->st))) return st;
            continue;
        }
        if ((st = status_error(c, w))) return st;
        done += k;
    }
    return NBG_OK;
}

extern "C" int nbg_advance(nbg_ctx* c, double dt, int64_t nsteps)
{
    NBG_RANGE("nbg_advance");
    if (!c) return NBG_ERR_ARG;
    NBG_ENTER(c);
    return advance_impl(c, dt, nsteps, true);
}

extern "C" int nbg_sync(nbg_ctx* c)
{
    NBG_RANGE("nbg_sync");
    if (!c) return NBG_ERR_ARG;
    NBG_ENTER(c);
    CK(cudaStreamSynchronize(c->stream), "sync");
    return NBG_OK;
}

extern "C" int nbg_run(nbg_ctx* c, double* u, double* v, double dt, int64_t nsteps, int64_t save_every,
                       double* traj_u, double* traj_v, nbg_run_stats* stats)
{
    NBG_RANGE("nbg_run");
    if (!c || !u || !v) return NBG_ERR_ARG;
    if (!(dt > 0.0) || nsteps < 0) return fail(c, NBG_ERR_ARG, "dt must be > 0 and nsteps >= 0");
    NBG_ENTER(c);
    int64_t launches0 = c->launches;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0), "event");
    CK(cudaEventCreate(&e1), "event");
    CK(cudaEventRecord(e0, c->stream), "event");
    unsigned long long builds0 = 0;
    int st;
    if ((st = nbg_set_state(c, u, v))) return st;
    // the step counter keys the Philox noise (Andersen, Langevin): it keeps
    // running across runs, so every run draws fresh noise, as the
    // reference's run_simulation does; nbg_set_step restarts or restores it
    const int64_t t0 = c->step;
    if (c->path == PATH_LIST) CK(cudaMemcpyAsync(&builds0, c->d.build_count, 8, cudaMemcpyDeviceToHost, c->stream), "builds");
    size_t fb = state_bytes(c);
    const int64_t n3 = 3 * c->cols;
    int64_t frame = 0;
    if (traj_u) memcpy(traj_u, u, fb);
    if (traj_v) memcpy(traj_v, v, fb);
    ++frame;
    // frames at the multiples of save_every are written by the steps into a
    // device buffer (up to RUN_FRAME_BYTES of them at a time) and copied out
    // once per segment; a last partial interval ends with the final state
    const bool traj = traj_u || traj_v;
    const int64_t aligned = traj && save_every > 0 ? nsteps / save_every : 0;
    int64_t cap = 0;
    if (aligned > 0) {
        cap = std::max<int64_t>(1, std::min<int64_t>(aligned, (int64_t)(RUN_FRAME_BYTES / (2 * fb))));
        if (c->frames_cap < cap) {
            if (c->frames) cudaFree(c->frames);
            c->frames = nullptr;
            c->frames_cap = 0;
            cudaError_t e = cudaMalloc(&c->frames, 2 * (size_t)cap * fb);
            if (e != cudaSuccess) {
                cudaGetLastError();
                c->frames = nullptr;
                return fail(c, NBG_ERR_NOMEM, "trajectory frames: cudaMalloc failed");
            }
            c->frames_cap = cap;
        }
    }
    int64_t done = 0;
    while (done < nsteps) {
        if (done / std::max<int64_t>(save_every, 1) < aligned) {
            const int64_t j0 = done / save_every + 1;  // the segment's first frame
            const int64_t nf = std::min<int64_t>(cap, aligned - (j0 - 1));
            const FrameSink h{c->frames, c->frames + (size_t)c->frames_cap * n3, save_every, j0, nf, t0};
            CK(cudaMemcpy(c->d.sink, &h, sizeof h, cudaMemcpyHostToDevice), "frame sink");
            c->sink_on = true;
            st = advance_impl(c, dt, nf * save_every);
            c->sink_on = false;
            if (st) return st;
            if (traj_u) CK(cudaMemcpyAsync(traj_u + j0 * n3, h.x, nf * fb, cudaMemcpyDeviceToHost, c->stream), "traj");
            if (traj_v) CK(cudaMemcpyAsync(traj_v + j0 * n3, h.v, nf * fb, cudaMemcpyDeviceToHost, c->stream), "traj");
            done += nf * save_every;
            frame = j0 + nf;
        } else {
            const int64_t k = nsteps - done;
            if ((st = advance_impl(c, dt, k))) return st;
            done += k;
            if (traj) {
                if (traj_u) CK(cudaMemcpyAsync(traj_u + frame * n3, c->st.x, fb, cudaMemcpyDeviceToHost, c->stream), "traj");
                if (traj_v) CK(cudaMemcpyAsync(traj_v + frame * n3, c->st.v, fb, cudaMemcpyDeviceToHost, c->stream), "traj");
                ++frame;
            }
        }
    }
    CK(cudaMemcpyAsync(u, c->st.x, fb, cudaMemcpyDeviceToHost, c->stream), "u download");
    CK(cudaMemcpyAsync(v, c->st.v, fb, cudaMemcpyDeviceToHost, c->stream), "v download");
    CK(cudaEventRecord(e1, c->stream), "event");
    CK(cudaStreamSynchronize(c->stream), "run sync");
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        unsigned long long builds1 = 0;
        if (c->path == PATH_LIST) cudaMemcpy(&builds1, c->d.build_count, 8, cudaMemcpyDeviceToHost);
        stats->steps = nsteps;
        stats->list_builds = (int64_t)(builds1 - builds0);
        stats->kernel_launches = c->launches - launches0;
        stats->device_ms = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return NBG_OK;
}

extern "C" int nbg_energy(nbg_ctx* c, const double* u, const double* v, nbg_energies* out)
{
    NBG_RANGE("nbg_energy");
    if (!c || !u || !v || !out) return NBG_ERR_ARG;
    if (c->nrep != 1) return fail(c, NBG_ERR_UNSUPPORTED, "energies are per system (create one context per replica)");
    NBG_ENTER(c);
    CK(cudaMemcpyAsync(c->ev.x, u, state_bytes(c), cudaMemcpyHostToDevice, c->stream), "u upload");
    CK(cudaMemcpyAsync(c->ev.v, v, state_bytes(c), cudaMemcpyHostToDevice, c->stream), "v upload");
    int st;
    if (c->path == PATH_LIST) resident_dirty(c);  // the list is rebuilt for u
    double h[7];
    for (int attempt = 0;; ++attempt) {
        if ((st = clear_status(c))) return st;
        if ((st = launch_energy(c, c->ev, h))) return st;
        unsigned w = 0;
        if ((st = read_status(c, &w))) return st;
        if (attempt < 6 && (w & (ST_CELL_OVERFLOW | ST_NBR_OVERFLOW)) && !(w & (ST_NONFINITE | ST_RANGE | ST_INDEX))) {
            if ((st = grow_lists(c, w))) return st;
            continue;
        }
        if ((st = status_error(c, w))) return st;
        break;
    }
    out->kinetic = h[0];
    out->lennard_jones = h[1];
    out->electrostatic = h[2];
    out->bonds = h[3];
    out->angles = h[4];
    out->gravity = h[5];
    out->potential = h[1] + h[2] + h[3] + h[4];
    out->total = out->kinetic + out->potential;
    out->temperature = h[6] / (c->d.kb * c->reps_h[0].ndf);
    return NBG_OK;
}

extern "C" int nbg_pair_list(nbg_ctx* c, const double* u, int32_t which, int32_t* pairs, int64_t cap, int64_t* count)
{
    NBG_RANGE("nbg_pair_list");
    if (!c || !u || !count || (which != NBG_POT_LJ && which != NBG_POT_EL)) return NBG_ERR_ARG;
    if (!(c->d.pots & which)) return fail(c, NBG_ERR_ARG, "potential not present");
    if (c->path == PATH_GRAVITY) return fail(c, NBG_ERR_UNSUPPORTED, "gravity has no pair list");
    NBG_ENTER(c);
    CK(cudaMemcpyAsync(c->ev.x, u, state_bytes(c), cudaMemcpyHostToDevice, c->stream), "u upload");
    resident_dirty(c);
    int st;
    // build the lists for u (forces_once packs and rebuilds)
    if ((st = forces_once(c, c->ev))) return st;
    int64_t per = c->path == PATH_LIST ? c->d.nbr_cap : c->n;
    int *dj = nullptr, *dc = nullptr;
    CK(cudaMallocAsync((void**)&dj, sizeof(int) * per * c->n, c->stream), "pairs scratch");
    CK(cudaMallocAsync((void**)&dc, sizeof(int) * c->n, c->stream), "pairs scratch");
    if ((st = launch_pairs(c, c->ev, which, dj, dc, per))) return st;
    std::vector<int> hj((size_t)per * c->n), hc(c->n);
    CK(cudaMemcpyAsync(hj.data(), dj, sizeof(int) * per * c->n, cudaMemcpyDeviceToHost, c->stream), "pairs copy");
    CK(cudaMemcpyAsync(hc.data(), dc, sizeof(int) * c->n, cudaMemcpyDeviceToHost, c->stream), "pairs copy");
    cudaFreeAsync(dj, c->stream);
    cudaFreeAsync(dc, c->stream);
    CK(cudaStreamSynchronize(c->stream), "pairs sync");
    unsigned w = 0;
    if ((st = read_status(c, &w))) return st;
    if ((st = status_error(c, w))) return st;
    int64_t total = 0;
    for (int64_t i = 0; i < c->n; ++i) {
        int m = std::min<int64_t>(hc[i], per);
        std::sort(hj.begin() + i * per, hj.begin() + i * per + m);
        for (int k = 0; k < m; ++k) {
            if (pairs && total < cap) {
                pairs[2 * total] = (int32_t)i;
                pairs[2 * total + 1] = hj[i * per + k];
            }
            ++total;
        }
    }
    *count = total;
    return NBG_OK;
}

// ---------------------------------------------------------------------
// learned short-range model of SPC/Fw water and r-RESPA (engine extension:
// the reference has neither a learned model nor a multiple-time-step
// integrator)
// ---------------------------------------------------------------------
static int ml_check(nbg_ctx* c)
{
    if (!c) return NBG_ERR_ARG;
    if (!c->ml_on) return fail(c, NBG_ERR_ARG, "learned model not enabled (call nbg_ml_enable)");
    NBG_ENTER(c);
    return NBG_OK;
}

static int ml_alloc_short(nbg_ctx* c, int scap)
{
    if (scap > 65535) return fail(c, NBG_ERR_CAPACITY, "short-list capacity above 65535");
    if (c->ml_snbr) dfree(c, c->ml_snbr);
    c->ml_snbr = nullptr;
    c->ml_scap = scap;
    return dalloc(c, &c->ml_snbr, (size_t)scap * c->n);
}

extern "C" int nbg_ml_param_count(void) { return ML_NPARAM; }

extern "C" int nbg_ml_enable(nbg_ctx* c)
{
    if (!c) return NBG_ERR_ARG;
    if (c->ml_on) return NBG_OK;
    if (c->d.kind != NBG_SYSTEM_WATER || c->path != PATH_LIST || c->nrep != 1 || c->d.bc != NBG_BC_CUBIC)
        return fail(c, NBG_ERR_UNSUPPORTED,
                    "the learned model needs one SPC/Fw water system on the Verlet-list path in a cubic box");
    NBG_ENTER(c);
    int st;
    if (ml_init_constants() != NBG_OK) return fail(c, NBG_ERR_CUDA, "learned-model constants");
    const int64_t n = c->n;
    for (int s = 0; s < 2; ++s) {
        if ((st = dalloc(c, &c->ml_theta[s], ML_NPARAM))) return st;
        if ((st = dalloc(c, &c->ml_w1[s], 64 * 128))) return st;
        if ((st = dalloc(c, &c->ml_w2[s], 128 * 128))) return st;
        if ((st = dalloc(c, &c->ml_ts.m1[s], ML_NTRAIN))) return st;
        if ((st = dalloc(c, &c->ml_ts.m2[s], ML_NTRAIN))) return st;
    }
    // unit normalisation until nbg_ml_normalize: sd = 1 (mean 0 from the zeroed allocation)
    {
        std::vector<float> th(ML_NPARAM, 0.0f);
        for (int k = 0; k < 64; ++k) th[ML_NTRAIN + 64 + k] = 1.0f;
        th[ML_NTRAIN + 129] = 1.0f;
        for (int s = 0; s < 2; ++s)
            CK(cudaMemcpyAsync(c->ml_theta[s], th.data(), sizeof(float) * ML_NPARAM, cudaMemcpyHostToDevice, c->stream),
               "ml params");
    }
    const double L = c->desc.box[0];
    const double rs = 0.6 + c->desc.skin;
    const double expect = 4.0 / 3.0 * M_PI * rs * rs * rs * (double)n / (L * L * L);
    const int scap = ((int)std::ceil(1.3 * expect + 32) + 7) / 8 * 8;
    if ((st = ml_alloc_short(c, scap))) return st;
    if ((st = dalloc(c, &c->ml_scnt, n))) return st;
    if ((st = dalloc(c, &c->ml_x, 64 * n))) return st;
    if ((st = dalloc(c, &c->ml_mom, 72 * n))) return st;
    if ((st = dalloc(c, &c->ml_dx, 64 * n))) return st;
    if ((st = dalloc(c, &c->ml_e, n))) return st;
    if ((st = dalloc(c, &c->ml_fq, 3 * n))) return st;
    if ((st = dalloc(c, &c->ml_fsr, 3 * n))) return st;
    if ((st = dalloc(c, &c->ml_esr, n))) return st;
    if ((st = dalloc(c, &c->ml_a_slow, 3 * c->cols))) return st;
    c->ml_judge_cap = 64;
    if ((st = dalloc(c, &c->ml_judge, 2 * c->ml_judge_cap))) return st;
    if ((st = launch_mlp_attrs(c))) return st;
    c->ml_on = true;
    if ((st = set_force_form(c))) return st;  // the learned kernels read the split positions every step
    for (int s = 0; s < 2; ++s)
        if ((st = launch_ml_pack(c, s))) return st;
    CK(cudaStreamSynchronize(c->stream), "ml enable sync");
    return NBG_OK;
}

extern "C" int nbg_ml_set_params(nbg_ctx* c, int32_t species, const float* theta)
{
    int st = ml_check(c);
    if (st) return st;
    if ((species != 0 && species != 1) || !theta) return fail(c, NBG_ERR_ARG, "species must be 0 (O) or 1 (H)");
    CK(cudaMemcpyAsync(c->ml_theta[species], theta, sizeof(float) * ML_NPARAM, cudaMemcpyHostToDevice, c->stream),
       "ml params upload");
    if ((st = launch_ml_pack(c, species))) return st;
    CK(cudaMemsetAsync(c->ml_ts.m1[species], 0, sizeof(float) * ML_NTRAIN, c->stream), "adam reset");
    CK(cudaMemsetAsync(c->ml_ts.m2[species], 0, sizeof(float) * ML_NTRAIN, c->stream), "adam reset");
    c->ml_adam_t[species] = 0;
    c->respa_valid = false;
    CK(cudaStreamSynchronize(c->stream), "ml params sync");
    return NBG_OK;
}

extern "C" int nbg_ml_get_params(nbg_ctx* c, int32_t species, float* theta)
{
    int st = ml_check(c);
    if (st) return st;
    if ((species != 0 && species != 1) || !theta) return fail(c, NBG_ERR_ARG, "species must be 0 (O) or 1 (H)");
    CK(cudaMemcpyAsync(theta, c->ml_theta[species], sizeof(float) * ML_NPARAM, cudaMemcpyDeviceToHost, c->stream),
       "ml params download");
    CK(cudaStreamSynchronize(c->stream), "ml params sync");
    return NBG_OK;
}

// splitmix64 (Steele, Lea & Flood 2014) and Box-Muller normals for the host-side initialisation
static uint64_t splitmix64(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static double host_normal(uint64_t& s)
{
    const double u1 = ((splitmix64(s) >> 11) + 1.0) * (1.0 / 9007199254740993.0);
    const double u2 = (splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
}

extern "C" int nbg_ml_init_params(nbg_ctx* c, uint64_t seed, double w1_scale)
{
    int st = ml_check(c);
    if (st) return st;
    for (int s = 0; s < 2; ++s) {
        std::vector<float> th(ML_NPARAM);
        CK(cudaMemcpyAsync(th.data(), c->ml_theta[s], sizeof(float) * ML_NPARAM, cudaMemcpyDeviceToHost, c->stream),
           "ml params download");
        CK(cudaStreamSynchronize(c->stream), "ml params sync");
        uint64_t r = seed * 2 + (uint64_t)s + 1;
        int o = 0;
        for (int k = 0; k < 64 * 128; ++k) th[o++] = (float)(w1_scale * host_normal(r) / 8.0);
        for (int k = 0; k < 128; ++k) th[o++] = 0.0f;
        for (int k = 0; k < 128 * 128; ++k) th[o++] = (float)(host_normal(r) / std::sqrt(128.0));
        for (int k = 0; k < 128; ++k) th[o++] = 0.0f;
        for (int k = 0; k < 128; ++k) th[o++] = (float)(host_normal(r) / std::sqrt(128.0));
        th[o++] = 0.0f;
        if ((st = nbg_ml_set_params(c, s, th.data()))) return st;
    }
    return NBG_OK;
}

// Short list, descriptors and (unless raw) the learned energies and forces
// of the packed positions of state s. pos: time index of the positions.
static int ml_forces(nbg_ctx* c, StepRef pos, bool force_short, bool raw)
{
    int st;
    if ((st = launch_short_list(c, pos, force_short))) return st;
    if ((st = launch_descriptor(c, raw))) return st;
    if (raw) return NBG_OK;
    if ((st = launch_mlp(c))) return st;
    return launch_ml_force(c);
}

// One-off evaluation at host positions u (scratch view), with capacity
// retries. what: 0 learned model, 1 raw descriptors only, 2 labels only.
static int ml_eval_once(nbg_ctx* c, const double* u, int what)
{
    CK(cudaMemcpyAsync(c->ev.x, u, state_bytes(c), cudaMemcpyHostToDevice, c->stream), "u upload");
    resident_dirty(c);
    c->respa_valid = false;
    for (int attempt = 0; attempt < 6; ++attempt) {
        int st;
        if ((st = clear_status(c))) return st;
        if ((st = launch_pack(c, c->ev))) return st;
        if ((st = launch_list_build(c, c->ev, true, StepRef{0, nullptr}))) return st;
        if (what == 2) {
            if ((st = launch_short_list(c, StepRef{0, nullptr}, true))) return st;
            if ((st = launch_sr_exact(c, c->ml_esr, c->ml_fsr))) return st;
        } else if ((st = ml_forces(c, StepRef{0, nullptr}, true, what == 1))) {
            return st;
        }
        unsigned w = 0;
        if ((st = read_status(c, &w))) return st;
        if (w & ST_FATAL) return status_error(c, w);
        if (w & (ST_CELL_OVERFLOW | ST_NBR_OVERFLOW | ST_SHORT_OVERFLOW)) {
            if ((w & (ST_CELL_OVERFLOW | ST_NBR_OVERFLOW)) && (st = grow_lists(c, w))) return st;
            if ((w & ST_SHORT_OVERFLOW) && (st = ml_alloc_short(c, c->ml_scap + c->ml_scap / 2 + 32))) return st;
            continue;
        }
        return NBG_OK;
    }
    return fail(c, NBG_ERR_CAPACITY, "list capacity could not be grown enough");
}

extern "C" int nbg_ml_descriptors(nbg_ctx* c, const double* u, int32_t standardised, float* desc)
{
    NBG_RANGE("nbg_ml_descriptors");
    int st = ml_check(c);
    if (st) return st;
    if (!u || !desc) return fail(c, NBG_ERR_ARG, "null argument");
    if ((st = ml_eval_once(c, u, standardised ? 0 : 1))) return st;
    CK(cudaMemcpyAsync(desc, c->ml_x, sizeof(float) * 64 * c->n, cudaMemcpyDeviceToHost, c->stream), "desc download");
    CK(cudaStreamSynchronize(c->stream), "desc sync");
    return NBG_OK;
}

extern "C" int nbg_ml_eval(nbg_ctx* c, const double* u, float* energies, double* forces)
{
    NBG_RANGE("nbg_ml_eval");
    int st = ml_check(c);
    if (st) return st;
    if (!u) return fail(c, NBG_ERR_ARG, "null positions");
    if ((st = ml_eval_once(c, u, 0))) return st;
    if (energies)
        CK(cudaMemcpyAsync(energies, c->ml_e, sizeof(float) * c->n, cudaMemcpyDeviceToHost, c->stream), "e download");
    if (forces) {
        if ((st = launch_ml_force_out(c, c->ev.a_new))) return st;
        CK(cudaMemcpyAsync(forces, c->ev.a_new, sizeof(double) * 3 * c->n, cudaMemcpyDeviceToHost, c->stream),
           "f download");
    }
    CK(cudaStreamSynchronize(c->stream), "eval sync");
    return NBG_OK;
}

extern "C" int nbg_ml_labels(nbg_ctx* c, const double* u, float* energies, float* forces)
{
    NBG_RANGE("nbg_ml_labels");
    int st = ml_check(c);
    if (st) return st;
    if (!u) return fail(c, NBG_ERR_ARG, "null positions");
    if ((st = ml_eval_once(c, u, 2))) return st;
    if (energies)
        CK(cudaMemcpyAsync(energies, c->ml_esr, sizeof(float) * c->n, cudaMemcpyDeviceToHost, c->stream), "e download");
    if (forces)
        CK(cudaMemcpyAsync(forces, c->ml_fsr, sizeof(float) * 3 * c->n, cudaMemcpyDeviceToHost, c->stream),
           "f download");
    CK(cudaStreamSynchronize(c->stream), "labels sync");
    return NBG_OK;
}

extern "C" int nbg_ml_reserve(nbg_ctx* c, int64_t frames)
{
    int st = ml_check(c);
    if (st) return st;
    if (frames < 1) return fail(c, NBG_ERR_ARG, "frames must be >= 1");
    for (int s = 0; s < 2; ++s) {
        const int64_t cap = frames * (s == 0 ? c->n / 3 : 2 * (c->n / 3));
        if (c->ml_X[s]) dfree(c, c->ml_X[s]);
        if (c->ml_Y[s]) dfree(c, c->ml_Y[s]);
        c->ml_X[s] = nullptr;
        c->ml_Y[s] = nullptr;
        if ((st = dalloc(c, &c->ml_X[s], (size_t)cap * 64))) return st;
        if ((st = dalloc(c, &c->ml_Y[s], (size_t)cap))) return st;
        c->ml_cap[s] = cap;
        c->ml_rows[s] = 0;
    }
    return NBG_OK;
}

extern "C" int nbg_ml_collect(nbg_ctx* c, int64_t* rows)
{
    NBG_RANGE("nbg_ml_collect");
    int st = ml_check(c);
    if (st) return st;
    if (!c->state_valid) return fail(c, NBG_ERR_ARG, "no resident state (call nbg_set_state)");
    if (!c->ml_X[0]) return fail(c, NBG_ERR_ARG, "no training set (call nbg_ml_reserve)");
    const int64_t per[2] = {c->n / 3, 2 * (c->n / 3)};
    if (c->ml_rows[0] + per[0] > c->ml_cap[0] || c->ml_rows[1] + per[1] > c->ml_cap[1])
        return fail(c, NBG_ERR_CAPACITY, "training set full");
    // evaluate on the resident positions through the scratch path
    std::vector<double> u(3 * (size_t)c->cols);
    CK(cudaMemcpyAsync(u.data(), c->st.x, state_bytes(c), cudaMemcpyDeviceToHost, c->stream), "u download");
    CK(cudaStreamSynchronize(c->stream), "collect sync");
    if ((st = ml_eval_once(c, u.data(), 1))) return st;
    if ((st = launch_sr_exact(c, c->ml_esr, nullptr))) return st;
    for (int s = 0; s < 2; ++s) {
        if ((st = launch_ml_collect(c, s, c->ml_rows[s]))) return st;
        c->ml_rows[s] += per[s];
    }
    CK(cudaStreamSynchronize(c->stream), "collect sync");
    if (rows) {
        rows[0] = c->ml_rows[0];
        rows[1] = c->ml_rows[1];
    }
    return NBG_OK;
}

extern "C" int nbg_ml_normalize(nbg_ctx* c)
{
    NBG_RANGE("nbg_ml_normalize");
    int st = ml_check(c);
    if (st) return st;
    if (c->ml_rows[0] < 2 || c->ml_rows[1] < 2) return fail(c, NBG_ERR_ARG, "training set holds fewer than 2 rows");
    for (int s = 0; s < 2; ++s)
        if ((st = launch_ml_stats(c, s))) return st;
    c->respa_valid = false;
    CK(cudaStreamSynchronize(c->stream), "normalize sync");
    return NBG_OK;
}

static int ml_scratch(nbg_ctx* c, int B)
{
    MLTrainScratch& s = c->ml_ts;
    if (s.B >= B) return NBG_OK;
    float** bufs[] = {&s.xs, &s.a1, &s.a2, &s.g1, &s.g2, &s.eo, &s.grad};
    for (float** p : bufs) {
        if (*p) dfree(c, *p);
        *p = nullptr;
    }
    if (s.idx) dfree(c, s.idx);
    if (s.loss) dfree(c, s.loss);
    s.idx = nullptr;
    s.loss = nullptr;
    int st;
    if ((st = dalloc(c, &s.idx, B))) return st;
    if ((st = dalloc(c, &s.xs, (size_t)B * 64))) return st;
    if ((st = dalloc(c, &s.a1, (size_t)B * 128))) return st;
    if ((st = dalloc(c, &s.a2, (size_t)B * 128))) return st;
    if ((st = dalloc(c, &s.g1, (size_t)B * 128))) return st;
    if ((st = dalloc(c, &s.g2, (size_t)B * 128))) return st;
    if ((st = dalloc(c, &s.eo, B))) return st;
    if ((st = dalloc(c, &s.grad, ML_NTRAIN))) return st;
    if ((st = dalloc(c, &s.loss, 1))) return st;
    s.B = B;
    return NBG_OK;
}

extern "C" int nbg_ml_train(nbg_ctx* c, int64_t steps, int32_t batch, double lr, uint64_t seed, double* loss)
{
    NBG_RANGE("nbg_ml_train");
    int st = ml_check(c);
    if (st) return st;
    if (steps < 0 || batch < 1 || !(lr > 0.0)) return fail(c, NBG_ERR_ARG, "steps >= 0, batch >= 1, lr > 0");
    if (c->ml_rows[0] < 1 || c->ml_rows[1] < 1) return fail(c, NBG_ERR_ARG, "empty training set");
    if ((st = ml_scratch(c, batch))) return st;
    // loss of the last min(steps, 100) batches per species
    const int64_t tail = std::min<int64_t>(steps, 100);
    for (int s = 0; s < 2; ++s) {
        CK(cudaMemsetAsync(c->ml_ts.loss, 0, sizeof(double), c->stream), "loss clear");
        for (int64_t t = 0; t < steps; ++t) {
            if (t == steps - tail) CK(cudaMemsetAsync(c->ml_ts.loss, 0, sizeof(double), c->stream), "loss clear");
            // cosine schedule over this call
            const double f = 0.5 * (1.0 + std::cos(M_PI * (double)t / (double)steps));
            c->ml_adam_t[s] += 1;
            if ((st = launch_ml_train_step(c, s, batch, seed * 2 + (uint64_t)s, (uint64_t)c->ml_adam_t[s],
                                           (float)(lr * f), c->ml_adam_t[s])))
                return st;
        }
        if ((st = launch_ml_pack(c, s))) return st;
        double l = 0.0;
        CK(cudaMemcpyAsync(&l, c->ml_ts.loss, sizeof(double), cudaMemcpyDeviceToHost, c->stream), "loss read");
        CK(cudaStreamSynchronize(c->stream), "train sync");
        if (loss) loss[s] = tail > 0 ? l / (double)tail : 0.0;
    }
    c->respa_valid = false;
    return NBG_OK;
}

extern "C" int nbg_ml_batch_gradient(nbg_ctx* c, int32_t species, const float* x, const float* y, int32_t B,
                                     float* grad, double* loss)
{
    int st = ml_check(c);
    if (st) return st;
    if ((species != 0 && species != 1) || !x || !y || !grad || B < 1) return fail(c, NBG_ERR_ARG, "bad arguments");
    if ((st = ml_scratch(c, B))) return st;
    float *dX = nullptr, *dY = nullptr;
    CK(cudaMallocAsync((void**)&dX, sizeof(float) * 64 * (size_t)B, c->stream), "batch alloc");
    CK(cudaMallocAsync((void**)&dY, sizeof(float) * (size_t)B, c->stream), "batch alloc");
    CK(cudaMemcpyAsync(dX, x, sizeof(float) * 64 * (size_t)B, cudaMemcpyHostToDevice, c->stream), "batch upload");
    CK(cudaMemcpyAsync(dY, y, sizeof(float) * (size_t)B, cudaMemcpyHostToDevice, c->stream), "batch upload");
    CK(cudaMemsetAsync(c->ml_ts.loss, 0, sizeof(double), c->stream), "loss clear");
    st = launch_ml_batch_grad(c, c->ml_theta[species], dX, dY, B);
    cudaFreeAsync(dX, c->stream);
    cudaFreeAsync(dY, c->stream);
    if (st) return st;
    CK(cudaMemcpyAsync(grad, c->ml_ts.grad, sizeof(float) * ML_NTRAIN, cudaMemcpyDeviceToHost, c->stream),
       "grad download");
    double l = 0.0;
    CK(cudaMemcpyAsync(&l, c->ml_ts.loss, sizeof(double), cudaMemcpyDeviceToHost, c->stream), "loss read");
    CK(cudaStreamSynchronize(c->stream), "grad sync");
    if (loss) *loss = l;
    return NBG_OK;
}

extern "C" int nbg_ml_rows(nbg_ctx* c, int64_t* rows)
{
    int st = ml_check(c);
    if (st) return st;
    if (!rows) return NBG_ERR_ARG;
    rows[0] = c->ml_rows[0];
    rows[1] = c->ml_rows[1];
    return NBG_OK;
}

// r-RESPA state of the resident positions: a_old = fast (bonded + learned)
// and ml_a_slow = slow (exact non-bonded - learned) accelerations.
// The fast non-bonded acceleration into a: learned (fixed-point forces, then
// converted) or exact short-range (written directly).
// Fast-force modes of r-RESPA: 0 the learned model, 1 the exact short-range
// force (the classical split), 2 none (bonded terms only: the integrator's
// own cost, a ceiling for any fast non-bonded model).
static int respa_inner_force(nbg_ctx* c, StepRef pos, bool force_short, int mode, double* a)
{
    if (mode == 1) return launch_sr_inner(c, pos, force_short, a);
    if (mode == 2) {
        CK(cudaMemsetAsync(a, 0, state_bytes(c), c->stream), "fast force clear");
        return NBG_OK;
    }
    int st = ml_forces(c, pos, force_short, false);
    if (st) return st;
    return launch_ml_accel(c, 0, a);
}

// a -= the fast non-bonded acceleration of the last respa_inner_force
static int respa_sub_fast(nbg_ctx* c, int mode, double* a)
{
    if (mode == 2) return NBG_OK;
    return mode == 1 ? launch_sr_accel(c, -1, a) : launch_ml_accel(c, -1, a);
}

static int respa_init(nbg_ctx* c, int exact)
{
    int st;
    const StateView& s = c->st;
    const StepRef pos{c->step, nullptr};
    if ((st = launch_pack(c, s))) return st;
    if ((st = launch_list_build(c, s, true, pos))) return st;
    c->steps_since_build = 0;
    if ((st = respa_inner_force(c, pos, true, exact, s.a_old))) return st;
    StateView sb = s;
    sb.a_new = s.a_old;
    if ((st = launch_bonded(c, sb))) return st;
    StateView ss = s;
    ss.a_new = c->ml_a_slow;
    if ((st = launch_force_list(c, ss))) return st;
    if ((st = respa_sub_fast(c, exact, c->ml_a_slow))) return st;
    if (c->d.therm == NBG_THERMO_BERENDSEN && (st = launch_temperature(c, s.v))) return st;  // T for the first kick
    c->respa_valid = true;
    c->respa_mode = exact;
    c->accel_valid = false;  // a_old no longer holds the velocity-Verlet acceleration
    c->T_valid = false;
    return NBG_OK;
}

// One outer step (Tuckerman, Berne & Martyna 1992): slow half kick, `inner`
// velocity-Verlet steps of the fast force, the exact force at the new
// positions (slow force and judge), slow half kick. sr.off: step index of
// the outer step's start, counted in inner steps.
static int respa_outer(nbg_ctx* c, double dt, int inner, StepRef sr, int exact)
{
    int st;
    const StateView& s = c->st;
    const double H = 0.5 * dt * inner;
    // Berendsen: every kick reduces the temperature of its output for the next one
    const bool berendsen = c->d.therm == NBG_THERMO_BERENDSEN;
    if ((st = launch_respa_kick(c, s.v, c->ml_a_slow, H))) return st;
    for (int m = 0; m < inner; ++m) {
        const StepRef pos{sr.off + m + 1, sr.base};
        if ((st = launch_drift(c, s, dt, pos))) return st;
        const bool force = rebuild_due(c, true);
        if ((st = launch_list_build(c, s, force, pos))) return st;
        c->steps_since_build = force ? 0 : c->steps_since_build + 1;
        if ((st = respa_inner_force(c, pos, force, exact, s.a_new))) return st;
        if ((st = launch_bonded(c, s))) return st;
        if ((st = launch_kick(c, s, dt, berendsen, false))) return st;
    }
    StateView ss = s;
    ss.a_new = c->ml_a_slow;
    if ((st = launch_force_list(c, ss))) return st;
    if ((st = respa_sub_fast(c, exact, c->ml_a_slow))) return st;
    if (exact == 0) {
        // r-RESPA error check: the learned against the exact short-range force at these positions
        if ((st = launch_sr_exact(c, nullptr, c->ml_fsr))) return st;
        if ((st = launch_ml_judge(c, StepRef{sr.off + inner, sr.base}, inner, c->ml_judge_cap))) return st;
    }
    return launch_respa_kick(c, s.v, c->ml_a_slow, H);
}

extern "C" int nbg_respa_run(nbg_ctx* c, double dt, int32_t inner, int64_t outer, double threshold, int32_t flags,
                             nbg_respa_stats* out)
{
    NBG_RANGE("nbg_respa_run");
    // (named `exact` for the fast-force mode: see respa_inner_force)
    const int exact = (flags & NBG_RESPA_NO_FAST_FORCE) ? 2 : (flags & NBG_RESPA_EXACT_SPLIT) ? 1 : 0;
    int st = ml_check(c);
    if (st) return st;
    if (!c->state_valid) return fail(c, NBG_ERR_ARG, "no resident state (call nbg_set_state)");
    if (!(dt > 0.0) || inner < 1 || outer < 0) return fail(c, NBG_ERR_ARG, "dt > 0, inner >= 1, outer >= 0");
    if (c->d.therm != NBG_THERMO_NULL && c->d.therm != NBG_THERMO_BERENDSEN)
        return fail(c, NBG_ERR_UNSUPPORTED, "r-RESPA supports no thermostat or Berendsen");
    nbg_respa_stats S{};
    c->accel_lists_valid = false;
    const int64_t chunk = c->ml_judge_cap;
    if ((st = ensure_backup(c))) return st;
    double* b_slow = c->bk + 9 * c->cols;  // the slow acceleration's slot of the backup
    auto done_with = [&](int code) {
        c->accel_valid = false;
        if (out) *out = S;
        return code;
    };
    if ((st = clear_status(c))) return done_with(st);
    int64_t done = 0;
    int retries = 0;
    std::vector<double> judge(2 * (size_t)chunk);
    while (done < outer) {
        const int64_t k = std::min<int64_t>(chunk, outer - done);
        if ((!c->respa_valid || c->respa_mode != exact) && (st = respa_init(c, exact))) return done_with(st);
        const int64_t step0 = c->step;
        const int64_t ssb0 = c->steps_since_build;
        const size_t sb = state_bytes(c);
        if ((st = backup_state(c, false))) return done_with(st);
        CK(cudaMemcpyAsync(b_slow, c->ml_a_slow, sb, cudaMemcpyDeviceToDevice, c->stream), "backup");
        CK(cudaMemsetAsync(c->ml_judge, 0, sizeof(double) * 2 * chunk, c->stream), "judge clear");
        for (int64_t o = 0; o < k && st == NBG_OK; ++o) {
            st = respa_outer(c, dt, inner, StepRef{c->step, nullptr}, exact);
            c->step += inner;
        }
        if (st) return done_with(st);
        unsigned w = 0;
        if ((st = read_status(c, &w))) return done_with(st);
        CK(cudaMemcpyAsync(judge.data(), c->ml_judge, sizeof(double) * 2 * chunk, cudaMemcpyDeviceToHost, c->stream),
           "judge read");
        CK(cudaStreamSynchronize(c->stream), "judge sync");
        auto restore = [&]() -> int {
            int rs = backup_state(c, true);
            if (rs) return rs;
            CK(cudaMemcpyAsync(c->ml_a_slow, b_slow, sb, cudaMemcpyDeviceToDevice, c->stream), "restore");
            c->step = step0;
            c->steps_since_build = ssb0;
            c->T_valid = false;
            return clear_status(c);
        };
        if (w & ST_FATAL) return done_with(status_error(c, w));
        if (w & (ST_CELL_OVERFLOW | ST_NBR_OVERFLOW | ST_SHORT_OVERFLOW)) {
            if (++retries > 6) return done_with(fail(c, NBG_ERR_CAPACITY, "list capacity could not be grown enough"));
            if ((w & (ST_CELL_OVERFLOW | ST_NBR_OVERFLOW)) && (st = grow_lists(c, w))) return done_with(st);
            if ((w & ST_SHORT_OVERFLOW) && (st = ml_alloc_short(c, c->ml_scap + c->ml_scap / 2 + 32)))
                return done_with(st);
            if ((st = restore())) return done_with(st);
            c->respa_valid = false;  // lists were reallocated: rebuild everything at the chunk start
            continue;
        }
        // r-RESPA error check: relative RMS error of the learned against the exact short-range force
        double jmax = 0.0, jsum = 0.0;
        for (int64_t o = 0; o < k; ++o) {
            const int64_t slot = ((step0 / inner + o + 1) % chunk + chunk) % chunk;
            const double num = judge[2 * slot], den = judge[2 * slot + 1];
            const double r = den > 0.0 ? std::sqrt(num / den) : (num > 0.0 ? INFINITY : 0.0);
            jmax = std::max(jmax, r);
            jsum += r;
        }
        if (threshold > 0.0 && !(jmax <= threshold)) {
            // fallback: the chunk again by plain velocity Verlet with the exact force
            if ((st = restore())) return done_with(st);
            c->respa_valid = false;
            c->accel_valid = false;
            if ((st = advance_impl(c, dt, k * inner))) return done_with(st);
            S.outer_fallback += k;
            S.judge_last = jmax;
        } else {
            S.outer_mts += k;
            S.judged += k;
            S.judge_mean += jsum;
            S.judge_max = std::max(S.judge_max, jmax);
            S.judge_last = jmax;
        }
        done += k;
    }
    if (S.judged > 0) S.judge_mean /= (double)S.judged;
    return done_with(NBG_OK);
}

extern "C" int nbg_set_thermostat_target(nbg_ctx* c, int32_t replica, double T)
{
    if (!c) return NBG_ERR_ARG;
    if (replica < 0 || replica >= c->nrep || !(T >= 0.0) || !std::isfinite(T))
        return fail(c, NBG_ERR_ARG, "replica in range and a finite T >= 0");
    NBG_ENTER(c);
    c->reps_h[replica].T0 = T;
    if (replica == 0) c->desc.thermo_T = T;
    c->baoab_dt = -1.0;  // BAOAB noise amplitude follows T0
    RepDev* rp = const_cast<RepDev*>(c->d.reps) + replica;
    CK(cudaMemcpyAsync(rp, &c->reps_h[replica], sizeof(RepDev), cudaMemcpyHostToDevice, c->stream), "replica upload");
    CK(cudaStreamSynchronize(c->stream), "replica sync");
    return NBG_OK;  // captured graphs read the replica table at run time
}

extern "C" int nbg_ml_kernel_times(nbg_ctx* c, int32_t reps, double* ms)
{
    int st = ml_check(c);
    if (st) return st;
    if (!c->state_valid || reps < 1 || !ms) return fail(c, NBG_ERR_ARG, "resident state, reps >= 1, ms[4]");
    const StepRef pos{c->step, nullptr};
    if ((st = launch_pack(c, c->st))) return st;
    if ((st = launch_list_build(c, c->st, true, pos))) return st;
    resident_dirty(c);
    cudaEvent_t ev[5];
    for (auto& e : ev) CK(cudaEventCreate(&e), "event");
    double acc[4] = {0, 0, 0, 0};
    for (int r = 0; r < reps && st == NBG_OK; ++r) {
        cudaEventRecord(ev[0], c->stream);
        st = launch_short_list(c, pos, true);
        cudaEventRecord(ev[1], c->stream);
        if (!st) st = launch_descriptor(c, false);
        cudaEventRecord(ev[2], c->stream);
        if (!st) st = launch_mlp(c);
        cudaEventRecord(ev[3], c->stream);
        if (!st) st = launch_ml_force(c);
        cudaEventRecord(ev[4], c->stream);
        cudaEventSynchronize(ev[4]);
        for (int k = 0; k < 4; ++k) {
            float t = 0.f;
            cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
            acc[k] += t;
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    if (st) return st;
    for (int k = 0; k < 4; ++k) ms[k] = acc[k] / reps;
    return NBG_OK;
}

// Autotuner of the Verlet-list force kernel: on the resident positions, time
// every lanes-per-atom form (a thread per atom with a column-major list, or
// 4 / 8 / 16 / 32 lanes per atom with a row-major list) over `reps` launches
// and keep the fastest for this context.
extern "C" int nbg_autotune(nbg_ctx* c, int32_t reps, int32_t* lpa_out, double* ms_out)
{
    NBG_RANGE("nbg_autotune");
    if (!c) return NBG_ERR_ARG;
    if (c->path != PATH_LIST) return fail(c, NBG_ERR_UNSUPPORTED, "autotuning applies to the Verlet-list path");
    if (!c->state_valid) return fail(c, NBG_ERR_ARG, "no resident state (call nbg_set_state)");
    NBG_ENTER(c);
    if (reps < 1) reps = 1;
    const int cands[5] = {1, 4, 8, 16, 32};
    const int keep = c->list_lpa;
    int best = keep;
    double best_ms = INFINITY;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0), "event");
    CK(cudaEventCreate(&e1), "event");
    int st = NBG_OK;
    for (int k = 0; k < 5 && st == NBG_OK; ++k) {
        c->list_lpa = cands[k];
        if ((st = set_force_form(c))) break;
        if ((st = clear_status(c))) break;
        if ((st = launch_pack(c, c->st))) break;
        if ((st = launch_list_build(c, c->st, true, StepRef{c->step, nullptr}))) break;
        if ((st = launch_force_list(c, c->st))) break;  // warm-up
        cudaEventRecord(e0, c->stream);
        for (int r = 0; r < reps && st == NBG_OK; ++r) st = launch_force_list(c, c->st);
        cudaEventRecord(e1, c->stream);
        if (st) break;
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
            st = cuda_fail(c, e, "autotune sync");
            break;
        }
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        unsigned w = 0;
        if ((st = read_status(c, &w))) break;
        if ((st = status_error(c, w))) break;
        const double ms = (double)t / reps;
        if (ms_out) ms_out[k] = ms;
        if (ms < best_ms) {
            best_ms = ms;
            best = cands[k];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->list_lpa = st == NBG_OK ? best : keep;
    const int st2 = set_force_form(c);  // (drops captured launches of the previous form)
    if (st == NBG_OK) st = st2;
    resident_dirty(c);  // the next step rebuilds the list in the chosen layout
    if (lpa_out) *lpa_out = c->list_lpa;
    return st;
}

// Autotuner of the persistent ensemble loop: every form (lanes per atom 4 or
// 8; 512, 768 or 1024 threads per replica; cells of rl over 3^3 or of rl/2
// over 5^3) runs `steps` steps from the resident state (lists built afresh,
// so every form pays one build), timed by CUDA events; the state and the
// step counter are put back after each, and the fastest form is kept.
extern "C" int nbg_ensemble_tune(nbg_ctx* c, int32_t steps, int32_t* form, double* ms_out)
{
    NBG_RANGE("nbg_ensemble_tune");
    if (!c) return NBG_ERR_ARG;
    NBG_ENTER(c);
    if (!c->ens_ok && !c->ens_tuned_off)
        return fail(c, NBG_ERR_UNSUPPORTED, "the batch does not run the persistent ensemble loop");
    if (!c->state_valid) return fail(c, NBG_ERR_ARG, "no resident state (call nbg_set_state)");
    if (steps < 1) steps = 1;
    int st;
    if (c->ens_tuned_off) {  // an earlier tuning chose the step graphs: every form is timed again
        c->ens_disabled = false;
        c->ens_tuned_off = false;
        if (!ensemble_plan(c)) return fail(c, NBG_ERR_UNSUPPORTED, "the batch no longer fits the ensemble loop");
    }
    if (!c->accel_valid && (st = init_accel(c))) return st;
    if ((st = ensure_backup(c))) return st;
    if ((st = backup_state(c, false))) return st;
    const double dt = c->baoab_dt > 0.0 ? c->baoab_dt : 0.005;
    if (c->baoab && c->baoab_dt <= 0.0) {
        for (int r = 0; r < c->nrep; ++r) {
            RepDev& R = c->reps_h[r];
            R.bc1 = std::exp(-R.tparam * dt);
            R.bsd = std::sqrt(1.0 - R.bc1 * R.bc1) * std::sqrt(c->d.kb * R.T0);
        }
        CK(cudaMemcpy(const_cast<RepDev*>(c->d.reps), c->reps_h.data(), sizeof(RepDev) * c->nrep,
                      cudaMemcpyHostToDevice), "replica upload");
        c->baoab_dt = dt;
    }
    const int64_t step0 = c->step;
    const int keep[3] = {c->ens_lpa, c->ens_threads, c->ens_cells};
    int best = -1;
    double best_ms = INFINITY;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0), "event");
    CK(cudaEventCreate(&e1), "event");
    static const int lanes_of[2] = {4, 8}, threads_of[3] = {512, 768, 1024};
    for (int f = 0; f < 12 && st == NBG_OK; ++f) {
        c->ens_lpa = lanes_of[f / 6];
        c->ens_threads = threads_of[(f / 2) % 3];
        c->ens_cells = 1 + f % 2;
        double ms = INFINITY;
        if (ensemble_plan(c)) {
            c->ens_lists_valid = false;
            if ((st = clear_status(c))) break;
            cudaEventRecord(e0, c->stream);
            if ((st = launch_ensemble(c, c->st, dt, steps, step0, c->d.status))) break;
            cudaEventRecord(e1, c->stream);
            unsigned w = 0;
            if ((st = read_status(c, &w))) break;
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            if (!(w & ST_FATAL)) ms = (double)t / steps;
            if ((st = backup_state(c, true))) break;
        }
        if (ms_out) ms_out[f] = ms;
        if (ms < best_ms) {
            best_ms = ms;
            best = f;
        }
    }
    // form 12: the per-step kernels of the whole batch in CUDA graphs, from
    // the same state, with the same full list build at its first step (one
    // untimed pass captures the graphs first)
    if (st == NBG_OK) {
        double ms = INFINITY;
        c->ens_ok = false;
        for (int pass = 0; pass < 2 && st == NBG_OK; ++pass) {
            c->step = step0;
            c->steps_since_build = -1;
            c->T_valid = false;
            cudaEventRecord(e0, c->stream);
            st = advance_impl(c, dt, steps, false);
            cudaEventRecord(e1, c->stream);
            float t = 0.f;
            if (st == NBG_OK && cudaEventSynchronize(e1) == cudaSuccess &&
                cudaEventElapsedTime(&t, e0, e1) == cudaSuccess && pass == 1)
                ms = (double)t / steps;
            int st3 = backup_state(c, true);
            if (st == NBG_OK) st = st3;
        }
        c->step = step0;
        c->ens_ok = true;
        if (ms_out) ms_out[12] = ms;
        if (st == NBG_OK && ms < best_ms) {
            best_ms = ms;
            best = 12;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st == NBG_OK && best == 12) {
        // the step graphs win: the batch leaves the loop (until tuned again)
        c->ens_lpa = keep[0];
        c->ens_threads = keep[1];
        c->ens_cells = keep[2];
        c->ens_ok = false;
        c->ens_disabled = true;
        c->ens_tuned_off = true;
        c->ens_lists_valid = false;
        c->steps_since_build = -1;
        int st2 = clear_status(c);
        if (form) form[0] = form[1] = form[2] = 0;
        return st2;
    }
    if (st == NBG_OK && best >= 0) {
        c->ens_lpa = lanes_of[best / 6];
        c->ens_threads = threads_of[(best / 2) % 3];
        c->ens_cells = 1 + best % 2;
    } else {
        c->ens_lpa = keep[0];
        c->ens_threads = keep[1];
        c->ens_cells = keep[2];
    }
    ensemble_plan(c);
    c->ens_lists_valid = false;
    c->steps_since_build = -1;
    int st2 = clear_status(c);
    if (st == NBG_OK) st = st2;
    if (form) {
        form[0] = c->ens_lpa;
        form[1] = c->ens_threads;
        form[2] = c->ens_cells == 2 ? 2 : 1;
    }
    return st;
}
