/*
 * oracle.c - FP64 CPU restatement of NBodySimulator.jl's hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the oracle the CUDA engine is tested against
 * (libnbg.so): only the tests, the smoke check and the benchmark's CPU-baseline
 * leg load it. It is never part of the product path.
 *
 * It restates, function by function and in the reference's loop order and
 * expression order, the Julia code of NBodySimulator.jl v1.15.0:
 *   src/boundary_conditions.jl:111-172   get_interparticle_distance
 *   src/basic_potentials.jl:240-433      pair / bonded accelerations
 *   src/thermostats.jl:76-128            Berendsen, md_temperature, Nose-Hoover
 *   src/nbody_to_ode.jl:263-433,460-680  marshalling, RHS closures, SDE drift
 *   src/nbody_simulation_result.jl:121-446,504-540  energies, Andersen
 * Build flags: -O3 -ffp-contract=off (Julia does not contract a*b+c into FMA).
 *
 * The velocity-Verlet and Euler-Maruyama integrators live in third-party
 * packages that are not part of the reference tree (OrdinaryDiffEqSymplecticRK
 * v2, StochasticDiffEq v7). They are restated from the published methods:
 *   VV:  u' = u + dt*v + dt^2/2*a;  a' = f(v, u');  v' = v + dt*(a/2 + a'/2)
 *   EM:  X' = X + dt*f(X) + g*dW,   dW ~ N(0, dt)
 * The velocity argument of f inside VV (the start-of-step velocity) and the
 * noise of the first-order SDE (sigma on velocity rows, 0 on position rows)
 * are this project's reading of those packages: parity there is unpinned by
 * the reference tree and only checked statistically by its thermostat tests.
 *
 * With NBG_FLAG_LANGEVIN_BAOAB the Langevin thermostat is integrated by BAOAB
 * (Leimkuhler & Matthews 2013) instead of Euler-Maruyama: an engine option
 * with no reference counterpart, restated here from the published scheme.
 *
 * Random numbers (Andersen collisions, Langevin noise) come from Philox4x32-10
 * (Salmon, Moraes, Dror, Shaw, SC'11) keyed by the descriptor's seed, with the
 * same counter layout as the CUDA engine; the reference uses Julia's unseeded
 * global RNG, so only statistical parity exists there.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/nbg.h"

static int g_threads = 1;

void oracle_set_threads(int n) { g_threads = n > 0 ? n : 1; }
int oracle_get_threads(void) { return g_threads; }

/* ------------------------------------------------------------------ */
/* minimum image: boundary_conditions.jl:111-172                        */
/* ------------------------------------------------------------------ */
typedef struct { double x, y, z, r, r2; } pairdist;

/* The reference's loops never end on coordinates that diverged to huge or
   infinite values; here each loop gives up after OR_MAX_ITERS passes (far
   beyond any physical input) and leaves the difference unwrapped. */
#define OR_MAX_ITERS (1 << 20)
int oracle_range_errors = 0;

static pairdist distance(const double* ri, const double* rj, const nbg_system_desc* d)
{
    pairdist p;
    double x = ri[0] - rj[0], y = ri[1] - rj[1], z = ri[2] - rj[2];
    long it = 0;
#define OR_LOOP(cond, stmt) \
    for (it = 0; (cond) && it < OR_MAX_ITERS; ++it) stmt; \
    if (it == OR_MAX_ITERS) oracle_range_errors++;
    if (d->bc == NBG_BC_CUBIC) { /* :138-165 */
        double size = d->box[0];
        double radius = 0.5 * size;
        OR_LOOP(x >= radius, x -= size)
        OR_LOOP(x < -radius, x += size)
        OR_LOOP(y >= radius, y -= size)
        OR_LOOP(y < -radius, y += size)
        OR_LOOP(z >= radius, z -= size)
        OR_LOOP(z < -radius, z += size)
    } else if (d->bc == NBG_BC_PERIODIC) { /* :111-136, maps into [lo, hi) */
        const double* b = d->box;
        OR_LOOP(x < b[0], x += b[1] - b[0])
        OR_LOOP(x >= b[1], x -= b[1] - b[0])
        OR_LOOP(y < b[2], y += b[3] - b[2])
        OR_LOOP(y >= b[3], y -= b[3] - b[2])
        OR_LOOP(z < b[4], z += b[5] - b[4])
        OR_LOOP(z >= b[5], z -= b[5] - b[4])
    }
#undef OR_LOOP
    p.x = x; p.y = y; p.z = z;
    p.r2 = x * x + y * y + z * z; /* rij[1]^2 + rij[2]^2 + rij[3]^2 */
    p.r = sqrt(p.r2);
    return p;
}

/* rdf's histogram (nbody_simulation_result.jl:664-709): in every frame, each
   unordered pair of the atoms idx[] (the reference's LJ participants) under
   cubic boundaries of side L, r from get_interparticle_distance, counted
   twice in bin = ceil(r / dr), dr = L / maxbin, when r^2 < (L/2)^2 and
   1 < bin <= maxbin. frames: nframes x (3 x ncols), the reference's layout.
   Threads split the pair rows and add integer-valued histograms, so the
   result does not depend on the thread count. */
void oracle_rdf_histogram(const double* frames, int64_t nframes, int64_t ncols, const int32_t* idx, int64_t nidx,
                          double L, int32_t maxbin, double* hist)
{
    nbg_system_desc d;
    memset(&d, 0, sizeof d);
    d.bc = NBG_BC_CUBIC;
    d.box[0] = L;
    const double dr = L / maxbin;
    const double half = 0.5 * L;
    const double half2 = half * half; /* (0.5 * pbc.L)^2 */
    for (int32_t b = 0; b < maxbin; ++b) hist[b] = 0.0;
    int nt = g_threads;
    double* part = (double*)calloc((size_t)nt * maxbin, sizeof(double));
#pragma omp parallel for num_threads(nt) schedule(dynamic, 16)
    for (int64_t a = 0; a < nidx; ++a) {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        double* h = part + (size_t)t * maxbin;
        for (int64_t f = 0; f < nframes; ++f) {
            const double* cc = frames + f * 3 * ncols;
            const double* ri = cc + 3 * (int64_t)idx[a];
            for (int64_t b = a + 1; b < nidx; ++b) {
                pairdist p = distance(ri, cc + 3 * (int64_t)idx[b], &d);
                if (p.r2 < half2) {
                    const double bin = ceil(p.r / dr);
                    if (bin > 1 && bin <= maxbin) h[(int64_t)bin - 1] += 2.0;
                }
            }
        }
    }
    for (int t = 0; t < nt; ++t)
        for (int32_t b = 0; b < maxbin; ++b) hist[b] += part[(size_t)t * maxbin + b];
    free(part);
}

static int is_water(const nbg_system_desc* d) { return d->kind == NBG_SYSTEM_WATER; }
static int64_t nh_cols(const nbg_system_desc* d) { return d->n + (d->thermostat == NBG_THERMO_NOSEHOOVER ? 1 : 0); }

/* n and Nc of get_degrees_of_freedom / obtain_data_for_*_thermostating
   (nbody_simulation_result.jl:152-164, nbody_to_ode.jl:392-433). For water
   the reference's n is 3 x molecules = atoms and Nc = 2 x molecules. */
static void dof(const nbg_system_desc* d, int64_t* N, int64_t* Nc)
{
    *N = d->n;
    *Nc = is_water(d) ? 2 * (d->n / 3) : 0;
}

/* LJ participants: all bodies (:290-300) or the O atoms of water (:302-314). */
static int lj_participant(const nbg_system_desc* d, int64_t i)
{
    return is_water(d) ? (i % 3 == 0) : 1;
}

/* Electrostatic exclusions (:316-351): self, or the whole molecule for water. */
static int el_excluded(const nbg_system_desc* d, int64_t i, int64_t j)
{
    return is_water(d) ? (i / 3 == j / 3) : (i == j);
}

/* ------------------------------------------------------------------ */
/* pair accelerations: basic_potentials.jl                              */
/* ------------------------------------------------------------------ */

/* pairwise_lennard_jones_acceleration! :240-272 */
static void lj_accel(double* dv, const double* rs, int64_t i, const nbg_system_desc* d)
{
    double sigma2 = d->lj_sigma * d->lj_sigma;
    double R2 = d->lj_cutoff * d->lj_cutoff;
    double f1 = 0.0, f2 = 0.0, f3 = 0.0;
    const double* ri = rs + 3 * i;
    for (int64_t j = 0; j < d->n; ++j) {
        if (!lj_participant(d, j) || j == i) continue;
        pairdist p = distance(ri, rs + 3 * j, d);
        if (p.r2 < R2) {
            double s6 = sigma2 / p.r2;
            s6 = s6 * s6 * s6;
            double s12 = s6 * s6;
            double factor = (2.0 * s12 - s6) / p.r2;
            f1 += factor * p.x;
            f2 += factor * p.y;
            f3 += factor * p.z;
        }
    }
    double coeff = 24.0 * d->lj_epsilon / d->mass[i];
    dv[0] += coeff * f1;
    dv[1] += coeff * f2;
    dv[2] += coeff * f3;
}

/* pairwise_electrostatic_acceleration! :274-304 */
static void el_accel(double* dv, const double* rs, int64_t i, const nbg_system_desc* d)
{
    double R2 = d->el_cutoff * d->el_cutoff;
    double f1 = 0.0, f2 = 0.0, f3 = 0.0;
    const double* ri = rs + 3 * i;
    const double* qs = d->charge;
    for (int64_t j = 0; j < d->n; ++j) {
        if (el_excluded(d, i, j)) continue;
        pairdist p = distance(ri, rs + 3 * j, d);
        if (p.r2 < R2) {
            double factor = qs[j] / (p.r * p.r2);
            f1 += factor * p.x;
            f2 += factor * p.y;
            f3 += factor * p.z;
        }
    }
    double coeff = d->el_k * qs[i] / d->mass[i];
    dv[0] += coeff * f1;
    dv[1] += coeff * f2;
    dv[2] += coeff * f3;
}

/* gravitational_acceleration! :306-331 (no boundary conditions, no cutoff) */
static void grav_accel(double* dv, const double* rs, int64_t i, const nbg_system_desc* d)
{
    double a1 = 0.0, a2 = 0.0, a3 = 0.0;
    const double* ri = rs + 3 * i;
    for (int64_t j = 0; j < d->n; ++j) {
        if (j == i) continue;
        const double* rj = rs + 3 * j;
        double x = ri[0] - rj[0], y = ri[1] - rj[1], z = ri[2] - rj[2];
        double nrm = sqrt(x * x + y * y + z * z);
        double factor = -d->grav_G * d->mass[j] / (nrm * nrm * nrm);
        a1 += factor * x;
        a2 += factor * y;
        a3 += factor * z;
    }
    dv[0] += a1;
    dv[1] += a2;
    dv[2] += a3;
}

/* magnetostatic_dipdip_acceleration! :333-365 */
static void mag_accel(double* dv, const double* rs, int64_t i, const nbg_system_desc* d)
{
    double f1 = 0.0, f2 = 0.0, f3 = 0.0;
    const double* mi = d->dipole + 3 * i;
    const double* ri = rs + 3 * i;
    for (int64_t j = 0; j < d->n; ++j) {
        if (j == i) continue;
        const double* mj = d->dipole + 3 * j;
        const double* rj = rs + 3 * j;
        double x = ri[0] - rj[0], y = ri[1] - rj[1], z = ri[2] - rj[2];
        double dd = x * x + y * y + z * z;
        double rij4 = dd * dd;
        double nrm = sqrt(dd);
        double r[3] = {x / nrm, y / nrm, z / nrm};
        double mir = mi[0] * r[0] + mi[1] * r[1] + mi[2] * r[2];
        double mij = mj[0] * r[0] + mj[1] * r[1] + mj[2] * r[2];
        double mimj = mi[0] * mj[0] + mi[1] * mj[1] + mi[2] * mj[2];
        double c[3];
        for (int k = 0; k < 3; ++k)
            c[k] = (mi[k] * mij + mj[k] * mir + r[k] * mimj - 5.0 * r[k] * mir * mij) / rij4;
        f1 += c[0];
        f2 += c[1];
        f3 += c[2];
    }
    double coeff = 3.0 * d->mag_mu_4pi / d->mass[i];
    dv[0] += coeff * f1;
    dv[1] += coeff * f2;
    dv[2] += coeff * f3;
}

/* harmonic_bond_potential_acceleration! :367-393 with the neighbourhoods of
   obtain_data_for_harmonic_bond_interaction (nbody_to_ode.jl:263-288):
   O -> (H1, H2), H -> (O). */
static void bond_accel(double* dv, const double* rs, int64_t i, const nbg_system_desc* d)
{
    int64_t o = 3 * (i / 3);
    int64_t nb[2];
    int cnt;
    if (i == o) { nb[0] = o + 1; nb[1] = o + 2; cnt = 2; }
    else { nb[0] = o; cnt = 1; }
    double f1 = 0.0, f2 = 0.0, f3 = 0.0;
    const double* ri = rs + 3 * i;
    for (int c = 0; c < cnt; ++c) {
        const double* rj = rs + 3 * nb[c];
        double x = ri[0] - rj[0], y = ri[1] - rj[1], z = ri[2] - rj[2];
        double r = sqrt(x * x + y * y + z * z);
        double dd = r - d->water_rOH;
        double factor = -dd * d->water_kb / r;
        f1 += factor * x;
        f2 += factor * y;
        f3 += factor * z;
    }
    double coeff = 1.0 / d->mass[i];
    dv[0] += coeff * f1;
    dv[1] += coeff * f2;
    dv[2] += coeff * f3;
}

static void cross3(const double* a, const double* b, double* c)
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
static double norm3(const double* a) { return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

/* valence_angle_potential_acceleration! :395-433, called with
   (a, b, c) = (H1, O, H2) by get_group_accelerating_function (nbody_to_ode.jl:244-261). */
/* The H1-O-H2 angle forces of molecule mol on its atoms a = H1, b = O,
   c = H2 (fa, fb, fc), then divided by the masses into dv. */
static void angle_forces(const double* rs, int64_t mol, const nbg_system_desc* d, double fa[3], double fb[3],
                         double fc[3])
{
    int64_t b = 3 * mol, a = b + 1, c = b + 2;
    const double *ra = rs + 3 * a, *rb = rs + 3 * b, *rc = rs + 3 * c;
    double rba[3], rbc[3], rcb[3], x[3], pa[3], pc[3];
    for (int k = 0; k < 3; ++k) {
        rba[k] = ra[k] - rb[k];
        rbc[k] = rc[k] - rb[k];
        rcb[k] = rb[k] - rc[k];
    }
    cross3(rba, rbc, x);
    cross3(rba, x, pa);
    cross3(rcb, x, pc);
    double npa = norm3(pa), npc = norm3(pc);
    for (int k = 0; k < 3; ++k) { pa[k] /= npa; pc[k] /= npc; }
    double nba = norm3(rba), nbc = norm3(rbc);
    double cosine = (rba[0] * rbc[0] + rba[1] * rbc[1] + rba[2] * rbc[2]) / (nba * nbc);
    if (cosine > 1.0) cosine = 1.0;
    else if (cosine < -1.0) cosine = -1.0;
    double ang = acos(cosine);
    double force = -d->water_ka * (ang - d->water_aHOH);
    for (int k = 0; k < 3; ++k) {
        fa[k] = pa[k] * force / nba;
        fc[k] = pc[k] * force / nbc;
        fb[k] = -(fa[k] + fc[k]);
    }
}

static void angle_accel(double* dv, const double* rs, int64_t mol, const nbg_system_desc* d)
{
    int64_t b = 3 * mol, a = b + 1, c = b + 2;
    double fa[3], fb[3], fc[3];
    angle_forces(rs, mol, d, fa, fb, fc);
    for (int k = 0; k < 3; ++k) {
        dv[3 * a + k] += fa[k] / d->mass[a];
        dv[3 * b + k] += fb[k] / d->mass[b];
        dv[3 * c + k] += fc[k] / d->mass[c];
    }
}

/* ------------------------------------------------------------------ */
/* thermostats.jl                                                       */
/* ------------------------------------------------------------------ */

/* md_temperature :87-91 over the first N columns */
double oracle_md_temperature(const double* v, const double* ms, double kb, int64_t N, int64_t Nc)
{
    double e = 0.0;
    for (int64_t i = 0; i < N; ++i) {
        double s = v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2];
        e += ms[i] * s;
    }
    return e / (kb * (double)(3 * N - Nc));
}

/* berendsen_acceleration! :76-83 */
static void berendsen(double* dv, const double* v, const nbg_system_desc* d)
{
    int64_t N, Nc;
    dof(d, &N, &Nc);
    double T = oracle_md_temperature(v, d->mass, d->kb, N, Nc);
    double gamma = 0.5 / d->thermo_param; /* BerendsenThermostat(T, tau): gamma = 0.5/tau, :72-74 */
    if (1.0 / T == INFINITY) {
        for (int64_t e = 0; e < 3 * d->n; ++e) dv[e] += gamma * v[e];
    } else {
        double s = gamma * (d->thermo_T / T - 1.0);
        for (int64_t e = 0; e < 3 * d->n; ++e) dv[e] += s * v[e];
    }
}

/* nosehoover_acceleration! :121-128; dv, u, v are 3 x (n+1) */
static void nosehoover(double* dv, const double* u, double* v, const nbg_system_desc* d)
{
    int64_t N, Nc;
    dof(d, &N, &Nc);
    int64_t zi = 3 * d->n;
    double zeta = u[zi];
    for (int64_t e = 0; e < 3 * (d->n + 1); ++e) dv[e] -= zeta * v[e];
    dv[zi] = 0.0; dv[zi + 1] = 0.0; dv[zi + 2] = 0.0;
    double T = oracle_md_temperature(v, d->mass, d->kb, N, Nc);
    double ndf = (double)(3 * N - Nc);
    double itau = 1.0 / d->thermo_param;
    v[zi] = itau * itau * (T / d->thermo_T - (ndf + 1.0) / ndf);
}

/* ------------------------------------------------------------------ */
/* RHS: soode_system! (nbody_to_ode.jl:474-488, water :502-532)          */
/* ------------------------------------------------------------------ */

static void potential_terms(double* a, const double* u, int64_t i, const nbg_system_desc* d)
{
    /* PotentialNBodySystem holds its potentials in a Dict; this restatement
       applies them in the fixed order LJ, electrostatic, gravity, magnetic. */
    if (d->potentials & NBG_POT_LJ) lj_accel(a, u, i, d);
    if (d->potentials & NBG_POT_EL) el_accel(a, u, i, d);
    if (d->potentials & NBG_POT_GRAV) grav_accel(a, u, i, d);
    if (d->potentials & NBG_POT_MAG) mag_accel(a, u, i, d);
}

/* Forces of the bodies only (no thermostat terms): dv[:, i] for i < n.
   For water the angle loop runs only when with_angles is set. */
static void body_accelerations_ex(double* dv, const double* u, const nbg_system_desc* d, int with_angles)
{
    int64_t n = d->n;
    if (!is_water(d)) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(g_threads)
        for (int64_t i = 0; i < n; ++i) {
            double* a = dv + 3 * i;
            a[0] = 0.0; a[1] = 0.0; a[2] = 0.0;
            potential_terms(a, u, i, d);
        }
        return;
    }
    int64_t nm = n / 3;
    /* O loop :503-512 (electrostatic, bond, LJ) */
#pragma omp parallel for schedule(dynamic, 16) num_threads(g_threads)
    for (int64_t m = 0; m < nm; ++m) {
        int64_t idx = 3 * m;
        double* a = dv + 3 * idx;
        a[0] = 0.0; a[1] = 0.0; a[2] = 0.0;
        el_accel(a, u, idx, d);
        bond_accel(a, u, idx, d);
        lj_accel(a, u, idx, d);
    }
    /* H loop :513-522 (electrostatic, bond) */
#pragma omp parallel for schedule(dynamic, 16) num_threads(g_threads)
    for (int64_t m = 0; m < nm; ++m) {
        for (int h = 1; h <= 2; ++h) {
            int64_t idx = 3 * m + h;
            double* a = dv + 3 * idx;
            a[0] = 0.0; a[1] = 0.0; a[2] = 0.0;
            el_accel(a, u, idx, d);
            bond_accel(a, u, idx, d);
        }
    }
    /* angle loop :523-527 */
    if (with_angles)
        for (int64_t m = 0; m < nm; ++m) angle_accel(dv, u, m, d);
}

static void body_accelerations(double* dv, const double* u, const nbg_system_desc* d)
{
    body_accelerations_ex(dv, u, d, 1);
}

int oracle_accel(const nbg_system_desc* d, double* dv, double* v, const double* u, double t)
{
    (void)t;
    body_accelerations(dv, u, d);
    if (d->thermostat == NBG_THERMO_BERENDSEN) berendsen(dv, v, d);
    else if (d->thermostat == NBG_THERMO_NOSEHOOVER) nosehoover(dv, u, v, d);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Philox4x32-10 and the engine's counter layout                        */
/* ------------------------------------------------------------------ */
static void philox4x32(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

/* Counter (atom, step lo, step hi, stream); key = seed. stream 0 gives the
   collision uniform, streams 1 and 2 give normals (Box-Muller). */
void oracle_philox(uint64_t seed, uint64_t atom, uint64_t step, uint32_t stream, uint32_t out[4])
{
    uint32_t c[4] = {(uint32_t)atom, (uint32_t)step, (uint32_t)(step >> 32), stream};
    philox4x32(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    memcpy(out, c, sizeof(c));
}

/* 53-bit uniform in [0,1) from two words */
static double u53(uint32_t a, uint32_t b)
{
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

/* Three standard normals for (atom, step). Box-Muller on 24-bit uniforms,
   the same uniforms the CUDA engine draws; evaluated here in double. */
void oracle_normals3(uint64_t seed, uint64_t atom, uint64_t step, double out[3])
{
    uint32_t w1[4], w2[4];
    oracle_philox(seed, atom, step, 1u, w1);
    oracle_philox(seed, atom, step, 2u, w2);
    const double two_pi = 6.283185307179586;
    double u1 = ((double)(w1[0] >> 8) + 1.0) * (1.0 / 16777216.0); /* (0, 1] */
    double u2 = (double)(w1[1] >> 8) * (1.0 / 16777216.0);        /* [0, 1) */
    double rr = sqrt(-2.0 * log(u1));
    out[0] = rr * cos(two_pi * u2);
    out[1] = rr * sin(two_pi * u2);
    double u3 = ((double)(w2[0] >> 8) + 1.0) * (1.0 / 16777216.0);
    double u4 = (double)(w2[1] >> 8) * (1.0 / 16777216.0);
    out[2] = sqrt(-2.0 * log(u3)) * cos(two_pi * u4);
}

double oracle_uniform(uint64_t seed, uint64_t atom, uint64_t step)
{
    uint32_t w[4];
    oracle_philox(seed, atom, step, 0u, w);
    return u53(w[0], w[1]);
}

/* Andersen affect! (nbody_simulation_result.jl:511-540) after step `step`. */
static void andersen(double* v, double dt, uint64_t step, const nbg_system_desc* d)
{
    double prob = d->thermo_param * dt; /* nu * (t - tprev) */
    for (int64_t i = 0; i < d->n; ++i) {
        if (oracle_uniform(d->seed, (uint64_t)i, step) < prob) {
            double m = is_water(d) ? d->mass[i] : d->mass[0];
            double vdev = sqrt(d->kb * d->thermo_T / m);
            double z[3];
            oracle_normals3(d->seed, (uint64_t)i, step, z);
            for (int k = 0; k < 3; ++k) v[3 * i + k] = vdev * z[k];
        }
    }
}

/* ------------------------------------------------------------------ */
/* integrators                                                          */
/* ------------------------------------------------------------------ */

/* Langevin drift of the first-order SDE (nbody_to_ode.jl:575-590 and the
   water version :612-666), velocity rows only: out = a(u) - friction. */
static void sde_velocity_drift_water(double* out, const double* u, const double* v, const nbg_system_desc* d);

static void sde_velocity_drift(double* out, const double* u, const double* v, const nbg_system_desc* d)
{
    if (is_water(d)) {
        sde_velocity_drift_water(out, u, v, d);
        return;
    }
    double g = d->thermo_param;
    int64_t n = d->n;
    body_accelerations(out, u, d);
    for (int64_t e = 0; e < 3 * n; ++e) out[e] -= g * v[e];
}

/* Water: the O loop subtracts gamma*v/m for O, H1 and H2, the H loop then
   zeroes the H rows before adding their forces, so only the O term stays
   (:629-647); the angle loop adds next (:649-657) and at the end every row
   loses gamma*v again (:664). */
static void sde_velocity_drift_water(double* out, const double* u, const double* v, const nbg_system_desc* d)
{
    double g = d->thermo_param;
    int64_t n = d->n;
    double mO = d->mass[0];
    body_accelerations_ex(out, u, d, 0);
    for (int64_t m = 0; m < n / 3; ++m)
        for (int k = 0; k < 3; ++k) {
            int64_t e = 3 * (3 * m) + k;
            out[e] -= g * v[e] / mO;
        }
    for (int64_t m = 0; m < n / 3; ++m) angle_accel(out, u, m, d);
    for (int64_t e = 0; e < 3 * n; ++e) out[e] -= g * v[e];
}

/* One Euler-Maruyama step at step index `step` (0-based). */
static void em_step(double* u, double* v, double* work, double dt, uint64_t step, const nbg_system_desc* d)
{
    int64_t n = d->n;
    sde_velocity_drift(work, u, v, d);
    double sq = sqrt(dt);
    double sig_body = sqrt(2.0 * d->thermo_param * d->kb * d->thermo_T / d->mass[0]);
    double sig_num = sqrt(2.0 * d->thermo_param * d->kb * d->thermo_T);
    for (int64_t i = 0; i < n; ++i) {
        double z[3];
        oracle_normals3(d->seed, (uint64_t)i, step, z);
        double sigma = is_water(d) ? sig_num / d->mass[i] : sig_body;
        for (int k = 0; k < 3; ++k) {
            int64_t e = 3 * i + k;
            double vn = v[e] + dt * work[e] + sigma * (sq * z[k]);
            u[e] = u[e] + dt * v[e];
            v[e] = vn;
        }
    }
}

/* BAOAB step (Leimkuhler & Matthews, Appl. Math. Res. eXpress 2013): B half
   kick, A half drift, O exact Ornstein-Uhlenbeck v = c1 v + c2 sqrt(kb T/m) z
   with c1 = exp(-gamma dt), c2 = sqrt(1 - c1^2), A half drift, forces, B half
   kick. Each atom uses its own mass. a holds the forces at u on entry and exit. */
static void baoab_step(double* u, double* v, double* a, double dt, uint64_t step, const nbg_system_desc* d)
{
    int64_t n = d->n;
    double c1 = exp(-d->thermo_param * dt);
    double c2 = sqrt(1.0 - c1 * c1);
    for (int64_t i = 0; i < n; ++i) {
        double z[3];
        oracle_normals3(d->seed, (uint64_t)i, step, z);
        double s = c2 * sqrt(d->kb * d->thermo_T / d->mass[i]);
        for (int k = 0; k < 3; ++k) {
            int64_t e = 3 * i + k;
            double vh = v[e] + (0.5 * dt) * a[e];
            double x = u[e] + (0.5 * dt) * vh;
            double vo = c1 * vh + s * z[k];
            u[e] = x + (0.5 * dt) * vo;
            v[e] = vo;
        }
    }
    body_accelerations(a, u, d);
    for (int64_t e = 0; e < 3 * n; ++e) v[e] = v[e] + (0.5 * dt) * a[e];
}

static void save_frame(double* traj, const double* x, int64_t cols, int64_t frame)
{
    if (traj) memcpy(traj + frame * 3 * cols, x, sizeof(double) * 3 * cols);
}

/* Velocity Verlet (published method; see header) with the RHS above, the
   Andersen callback after every step, or Euler-Maruyama for Langevin.
   u, v hold 3 x cols doubles (cols = n, or n+1 with Nose-Hoover). Frames are
   saved at step 0, every save_every steps, and at the end. Returns frames. */
int64_t oracle_run(const nbg_system_desc* d, double* u, double* v, double dt, int64_t nsteps,
                   int64_t save_every, double* traj_u, double* traj_v)
{
    int64_t cols = nh_cols(d);
    size_t bytes = sizeof(double) * 3 * cols;
    double* a = (double*)calloc(3 * cols, sizeof(double));
    double* an = (double*)calloc(3 * cols, sizeof(double));
    int64_t frame = 0;
    save_frame(traj_u, u, cols, frame);
    save_frame(traj_v, v, cols, frame);
    ++frame;
    if (d->thermostat == NBG_THERMO_LANGEVIN && (d->flags & NBG_FLAG_LANGEVIN_BAOAB)) {
        body_accelerations(a, u, d);
        for (int64_t s = 0; s < nsteps; ++s) {
            baoab_step(u, v, a, dt, (uint64_t)s, d);
            if ((save_every > 0 && (s + 1) % save_every == 0) || s + 1 == nsteps) {
                save_frame(traj_u, u, cols, frame);
                save_frame(traj_v, v, cols, frame);
                ++frame;
            }
        }
        free(a);
        free(an);
        return frame;
    }
    if (d->thermostat == NBG_THERMO_LANGEVIN) {
        for (int64_t s = 0; s < nsteps; ++s) {
            em_step(u, v, a, dt, (uint64_t)s, d);
            if ((save_every > 0 && (s + 1) % save_every == 0) || s + 1 == nsteps) {
                save_frame(traj_u, u, cols, frame);
                save_frame(traj_v, v, cols, frame);
                ++frame;
            }
        }
        free(a);
        free(an);
        return frame;
    }
    oracle_accel(d, a, v, u, 0.0);
    double dtsq = dt * dt;
    for (int64_t s = 0; s < nsteps; ++s) {
        for (int64_t e = 0; e < 3 * cols; ++e) u[e] = u[e] + dt * v[e] + dtsq * (0.5 * a[e]);
        oracle_accel(d, an, v, u, 0.0);
        for (int64_t e = 0; e < 3 * cols; ++e) v[e] = v[e] + dt * (0.5 * a[e] + 0.5 * an[e]);
        memcpy(a, an, bytes);
        if (d->thermostat == NBG_THERMO_ANDERSEN) andersen(v, dt, (uint64_t)s, d);
        if ((save_every > 0 && (s + 1) % save_every == 0) || s + 1 == nsteps) {
            save_frame(traj_u, u, cols, frame);
            save_frame(traj_v, v, cols, frame);
            ++frame;
        }
    }
    free(a);
    free(an);
    return frame;
}

/* ------------------------------------------------------------------ */
/* energies: nbody_simulation_result.jl:209-446                         */
/* ------------------------------------------------------------------ */

/* kinetic_energy :209-212 */
double oracle_kinetic_energy(const double* v, const double* ms, int64_t n)
{
    double e = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        double s = v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2];
        e += s * (ms[i] / 2.0);
    }
    return e;
}

/* lennard_jones_potential :293-319 (r^2 clamped to R^2 beyond the cutoff) */
static double lj_energy(const double* rs, const nbg_system_desc* d)
{
    double sigma2 = d->lj_sigma * d->lj_sigma, R2 = d->lj_cutoff * d->lj_cutoff;
    double e = 0.0;
#pragma omp parallel for reduction(+ : e) schedule(dynamic, 16) num_threads(g_threads)
    for (int64_t i = 0; i < d->n; ++i) {
        if (!lj_participant(d, i)) continue;
        for (int64_t j = i + 1; j < d->n; ++j) {
            if (!lj_participant(d, j)) continue;
            pairdist p = distance(rs + 3 * i, rs + 3 * j, d);
            double r2 = p.r2;
            if (!(r2 < R2)) r2 = R2;
            double s6 = sigma2 / r2;
            s6 = s6 * s6 * s6;
            e += (s6 * s6 - s6);
        }
    }
    return 4.0 * d->lj_epsilon * e;
}

/* electrostatic_potential :321-351 */
static double el_energy(const double* rs, const nbg_system_desc* d)
{
    double R2 = d->el_cutoff * d->el_cutoff;
    const double* qs = d->charge;
    double e = 0.0;
#pragma omp parallel for reduction(+ : e) schedule(dynamic, 16) num_threads(g_threads)
    for (int64_t i = 0; i < d->n; ++i) {
        double ei = 0.0;
        for (int64_t j = i + 1; j < d->n; ++j) {
            if (el_excluded(d, i, j)) continue;
            pairdist p = distance(rs + 3 * i, rs + 3 * j, d);
            if (p.r2 < R2) ei += qs[j] / p.r;
            else ei += qs[j] / d->el_cutoff;
        }
        e += ei * qs[i];
    }
    return e * d->el_k;
}

/* harmonic_bonds_potential :353-372: every directed bond, / 4 */
static double bond_energy(const double* rs, const nbg_system_desc* d)
{
    double e = 0.0;
    for (int64_t i = 0; i < d->n; ++i) {
        int64_t o = 3 * (i / 3);
        int64_t nb[2];
        int cnt;
        if (i == o) { nb[0] = o + 1; nb[1] = o + 2; cnt = 2; }
        else { nb[0] = o; cnt = 1; }
        for (int c = 0; c < cnt; ++c) {
            const double *ri = rs + 3 * i, *rj = rs + 3 * nb[c];
            double x = ri[0] - rj[0], y = ri[1] - rj[1], z = ri[2] - rj[2];
            double dd = sqrt(x * x + y * y + z * z) - d->water_rOH;
            e += dd * dd * d->water_kb;
        }
    }
    return e / 4.0;
}

/* valence_angle_harmonic_potential :374-397 (no clamp of the cosine) */
static double angle_energy(const double* rs, const nbg_system_desc* d)
{
    double e = 0.0;
    for (int64_t m = 0; m < d->n / 3; ++m) {
        const double *rb = rs + 9 * m, *ra = rb + 3, *rc = rb + 6;
        double rba[3], rbc[3];
        for (int k = 0; k < 3; ++k) { rba[k] = ra[k] - rb[k]; rbc[k] = rc[k] - rb[k]; }
        double ang = acos((rba[0] * rbc[0] + rba[1] * rbc[1] + rba[2] * rbc[2]) / (norm3(rba) * norm3(rbc)));
        double dd = ang - d->water_aHOH;
        e += d->water_ka * dd * dd;
    }
    return e / 2.0;
}

/* -G sum_{i<j} m_i m_j / r_ij (this project's definition; the reference has none) */
static double grav_energy(const double* rs, const nbg_system_desc* d)
{
    double e = 0.0;
#pragma omp parallel for reduction(+ : e) schedule(dynamic, 16) num_threads(g_threads)
    for (int64_t i = 0; i < d->n; ++i) {
        double ei = 0.0;
        for (int64_t j = i + 1; j < d->n; ++j) {
            const double *ri = rs + 3 * i, *rj = rs + 3 * j;
            double x = ri[0] - rj[0], y = ri[1] - rj[1], z = ri[2] - rj[2];
            ei += d->mass[j] / sqrt(x * x + y * y + z * z);
        }
        e += ei * d->mass[i];
    }
    return -d->grav_G * e;
}

int oracle_energy(const nbg_system_desc* d, const double* u, const double* v, nbg_energies* out)
{
    memset(out, 0, sizeof(*out));
    out->kinetic = oracle_kinetic_energy(v, d->mass, d->n);
    if (is_water(d)) {
        out->lennard_jones = lj_energy(u, d);
        out->electrostatic = el_energy(u, d);
        out->bonds = bond_energy(u, d);
        out->angles = angle_energy(u, d);
    } else {
        if (d->potentials & NBG_POT_LJ) out->lennard_jones = lj_energy(u, d);
        if (d->potentials & NBG_POT_EL) out->electrostatic = el_energy(u, d);
        if (d->potentials & NBG_POT_GRAV) out->gravity = grav_energy(u, d);
    }
    /* potential_energy (:239-291) in the reference's order; gravity stays
       outside it, as in the reference. */
    out->potential = out->lennard_jones + out->electrostatic + out->bonds + out->angles;
    out->total = out->kinetic + out->potential;
    int64_t N, Nc;
    dof(d, &N, &Nc);
    out->temperature = oracle_md_temperature(v, d->mass, d->kb, N, Nc);
    return 0;
}

/* The reference's pair set for one potential: ordered (i, j), j != i, with
   r^2 < R^2 (basic_potentials.jl:253-258 LJ, :288-292 electrostatic). */
int64_t oracle_pair_list(const nbg_system_desc* d, const double* u, int32_t which, int32_t* pairs, int64_t cap)
{
    int64_t cnt = 0;
    double R = which == NBG_POT_LJ ? d->lj_cutoff : d->el_cutoff;
    double R2 = R * R;
    for (int64_t i = 0; i < d->n; ++i) {
        if (which == NBG_POT_LJ && !lj_participant(d, i)) continue;
        for (int64_t j = 0; j < d->n; ++j) {
            if (which == NBG_POT_LJ) {
                if (!lj_participant(d, j) || j == i) continue;
            } else if (el_excluded(d, i, j)) {
                continue;
            }
            pairdist p = distance(u + 3 * i, u + 3 * j, d);
            if (p.r2 < R2) {
                if (cnt < cap) { pairs[2 * cnt] = (int32_t)i; pairs[2 * cnt + 1] = (int32_t)j; }
                ++cnt;
            }
        }
    }
    return cnt;
}

/* Accelerations of a subset of atoms [i0, i1) (bench CPU-baseline sample of
   the all-pairs work, and the sampled parity checks at full size; same
   per-atom loops as body_accelerations). For water, with i0 and i1 on
   molecule boundaries the angle terms (:526-531) of the molecules inside are
   added too, so the rows equal body_accelerations' rows. */
void oracle_partial_accel(const nbg_system_desc* d, const double* u, double* dv, int64_t i0, int64_t i1)
{
#pragma omp parallel for schedule(dynamic, 4) num_threads(g_threads)
    for (int64_t i = i0; i < i1; ++i) {
        double* a = dv + 3 * (i - i0);
        a[0] = 0.0; a[1] = 0.0; a[2] = 0.0;
        if (is_water(d)) {
            el_accel(a, u, i, d);
            bond_accel(a, u, i, d);
            if (i % 3 == 0) lj_accel(a, u, i, d);
        } else {
            potential_terms(a, u, i, d);
        }
    }
    if (is_water(d) && i0 % 3 == 0 && i1 % 3 == 0) {
        for (int64_t m = i0 / 3; m < i1 / 3; ++m) {
            double fa[3], fb[3], fc[3];
            angle_forces(u, m, d, fa, fb, fc);
            double* ab = dv + 3 * (3 * m - i0);
            for (int k = 0; k < 3; ++k) {
                ab[3 + k] += fa[k] / d->mass[3 * m + 1];
                ab[k] += fb[k] / d->mass[3 * m];
                ab[6 + k] += fc[k] / d->mass[3 * m + 2];
            }
        }
    }
}
