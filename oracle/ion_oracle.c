/*
 * ion_oracle.c -- TEST INFRASTRUCTURE: the CPU oracle.  Not product code;
 * only tests, the smoke check and the benchmark's CPU-baseline leg use it.
 *
 * A restatement, in plain C, of IonSolver's single-domain timestep
 * algorithm (the reference is Rust + OpenCL C; every function below cites
 * the reference lines it follows).  Compiled twice by oracle/build.py:
 *
 *   ORC_REAL=float  : the reference's arithmetic, operation for operation,
 *                     with the reference's FP16S/FP16C DDF storage codecs.
 *                     Built with -ffp-contract=off, so a*b+c is two
 *                     roundings unless the reference itself calls fma().
 *   ORC_REAL=double : the same formulas in double precision with double
 *                     storage (no 16-bit codecs): the FP64 accuracy oracle.
 *
 * Deliberate choices:
 *   - LOD charge/velocity bins are accumulated in ascending cell order, the
 *     order a sequential run of the reference's float atomics produces
 *     (sim_kernels.cl:666-677); a GPU run of the reference has no fixed order.
 *   - Only one domain (d_x=d_y=d_z=1), as on the path being replaced.
 *   - D3Q27 is rejected: the reference's get_device_defines emits no DEF_WC
 *     for it (src/lbm/domain.rs:766-768), so its kernels do not build.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

#include "ionsolver.h"

#ifndef ORC_REAL
#define ORC_REAL float
#endif
typedef ORC_REAL R;

#ifdef ORC_PREC_F32
#define RFMA fmaf
#define RSQRT sqrtf
#define RMIN fminf
#define RMAX fmaxf
#define THIRD_F 0.33333334f      /* literal of sim_kernels.cl:369-375 */
#define CS_F 0.57735027f         /* DEF_C, src/lbm/domain.rs:807 */
#else
#define RFMA fma
#define RSQRT sqrt
#define RMIN fmin
#define RMAX fmax
#define THIRD_F (1.0 / 3.0)
#define CS_F 0.57735026918962576
#endif

/* flag bits, src/lbm/domain.rs:819-828 */
#define F_S 0x01u
#define F_E 0x02u
#define F_C 0x04u
#define F_F 0x08u
#define F_M 0x10u
#define F_BO 0x1Fu

/* ------------------------------------------------------------------------
 * Velocity sets: direction vectors and weight classes
 * (sim_kernels.cl:326-365; weights from src/lbm/domain.rs:757-768).
 * Directions come in +/- pairs (1,2), (3,4), ...
 * ---------------------------------------------------------------------- */
typedef struct {
    int q, dims;
    signed char c[19][3];
    unsigned char wc[19]; /* 0 = centre, 1 = straight, 2 = edge/corner */
} vset;

static const vset VS_D2Q9 = {9, 2,
    {{0,0,0},{1,0,0},{-1,0,0},{0,1,0},{0,-1,0},{1,1,0},{-1,-1,0},{1,-1,0},{-1,1,0}},
    {0,1,1,1,1,2,2,2,2}};
static const vset VS_D3Q15 = {15, 3,
    {{0,0,0},{1,0,0},{-1,0,0},{0,1,0},{0,-1,0},{0,0,1},{0,0,-1},{1,1,1},{-1,-1,-1},
     {1,1,-1},{-1,-1,1},{1,-1,1},{-1,1,-1},{-1,1,1},{1,-1,-1}},
    {0,1,1,1,1,1,1,2,2,2,2,2,2,2,2}};
static const vset VS_D3Q19 = {19, 3,
    {{0,0,0},{1,0,0},{-1,0,0},{0,1,0},{0,-1,0},{0,0,1},{0,0,-1},{1,1,0},{-1,-1,0},
     {1,0,1},{-1,0,-1},{0,1,1},{0,-1,-1},{1,-1,0},{-1,1,0},{1,0,-1},{-1,0,1},{0,1,-1},{0,-1,1}},
    {0,1,1,1,1,1,1,2,2,2,2,2,2,2,2,2,2,2,2}};

/* ------------------------------------------------------------------------
 * 16-bit DDF storage codecs (float build only)
 * FP16S: scaled IEEE half, src/lbm/domain.rs:773-776 (vload_half(o,p)*2^-15,
 *        vstore_half_rte(x*2^15)).
 * FP16C: 1-4-11 custom format, sim_kernels.cl:79-90.
 * ---------------------------------------------------------------------- */
static uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

static float ieee_half_to_float(uint16_t h) {
    uint32_t s = (uint32_t)(h & 0x8000u) << 16, e = (h >> 10) & 31u, m = h & 1023u;
    if (e == 0u) { float v = ldexpf((float)m, -24); return s ? -v : v; }
    if (e == 31u) return u2f(s | 0x7F800000u | (m << 13) | (m ? 0x400000u : 0u));
    return u2f(s | ((e + 112u) << 23) | (m << 13));
}
static uint16_t ieee_float_to_half_rne(float f) {
    uint32_t x = f2u(f), s = (x >> 16) & 0x8000u, ax = x & 0x7FFFFFFFu;
    if (ax >= 0x7F800000u) return (uint16_t)(s | (ax > 0x7F800000u ? (0x7E00u | ((ax >> 13) & 1023u)) : 0x7C00u));
    if (ax >= 0x477FF000u) return (uint16_t)(s | 0x7C00u);
    if (ax >= 0x38800000u) { uint32_t r = ax - 0x38000000u; r += 0x0FFFu + ((r >> 13) & 1u); return (uint16_t)(s | (r >> 13)); }
    if (ax <= 0x33000000u) return (uint16_t)s;
    {
        uint32_t e = ax >> 23, m = (ax & 0x7FFFFFu) | 0x800000u, sh = 126u - e;
        uint32_t r = m >> sh, rem = m & ((1u << sh) - 1u), hw = 1u << (sh - 1u);
        if (rem > hw || (rem == hw && (r & 1u))) r++;
        return (uint16_t)(s | r);
    }
}
/* FP16C encode: round by adding 2^11 to the float's bit pattern, then keep
 * 4 exponent bits (bias 15) and 11 mantissa bits; small magnitudes become
 * 1-4-11 denormals, anything below goes to signed zero. */
/* NaN model: 0 = the host's NaN bit patterns (as the reference kernels
 * compiled for this host produce them); 1 = every NaN reaching the FP16C
 * encoder is the canonical quiet NaN 0x7FFFFFFF, the pattern NVIDIA GPUs
 * give NaN results (the GPU implementation's rule). */
static int g_canonical_nan = 0;
void orc_set_nan_model(int canonical) { g_canonical_nan = canonical != 0; }
static uint16_t fp16c_encode(float x) {
    const uint32_t xb = f2u(x);
    const uint32_t b = ((g_canonical_nan && (xb & 0x7FFFFFFFu) > 0x7F800000u) ? 0x7FFFFFFFu : xb) + 0x800u;
    const uint32_t e = (b & 0x7F800000u) >> 23, m = b & 0x007FFFFFu;
    uint32_t out = (b & 0x80000000u) >> 16;
    if (e > 112u) out |= (((e - 112u) << 11) & 0x7800u) | (m >> 12);
    else if (e > 100u) out |= (((0x007FF800u + m) >> (124u - e)) + 1u) >> 1;
    return (uint16_t)out;
}
static float fp16c_decode(uint16_t x) {
    const uint32_t e = (x & 0x7800u) >> 11, m = (uint32_t)(x & 0x07FFu) << 12;
    uint32_t out = (uint32_t)(x & 0x8000u) << 16;
    if (e != 0u) {
        out |= ((e + 112u) << 23) | m;
    } else if (m != 0u) {
        uint32_t lead = 31u; /* position of the highest set bit of m */
        while (!((m >> lead) & 1u)) lead--;
        out |= ((lead + 90u) << 23) | ((m << (23u - lead)) & 0x007FF000u);
    }
    return u2f(out);
}

/* ------------------------------------------------------------------------
 * handle
 * ---------------------------------------------------------------------- */
typedef struct {
    ion_config cfg;
    const vset* vs;
    uint32_t nx, ny, nz;
    uint64_t n;
    uint32_t n_lod_own, depth;
    uint64_t t;
    /* constants (get_device_defines, src/lbm/domain.rs:786-858) */
    R w, ke, kmu, kmu0, kkge, wq, wgt[3];
    R kkbme, keabs; /* SUBGRID_ECR (domain.rs:850-854) */
    /* DDF storage: R (f32/f64) or uint16 (FP16S/FP16C, float build only) */
    int ft; /* storage codec: 0 FP16S, 1 FP16C, 2 native */
    void *fi, *fqi, *ei, *eti;
    R *rho, *u, *F, *e_stat, *b_stat, *e_dyn, *b_dyn, *qf, *qu_lod, *e_var, *et;
    uint8_t* flags;
    size_t e_dyn_count;
    /* per-cell LOD contributions of the current step */
    R* lodc;
    uint8_t* lodm;
    /* background electron density of the finite-plasma start (0: the
     * reference's start, electron gas at density 0) */
    R rho_e0;
} orc;

static int g_threads = 1;
void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }

static R ld(const orc* h, const void* p, uint64_t i) {
#ifdef ORC_PREC_F32
    if (h->ft == ION_FP16S) return ieee_half_to_float(((const uint16_t*)p)[i]) * 3.0517578E-5f;
    if (h->ft == ION_FP16C) return fp16c_decode(((const uint16_t*)p)[i]);
#endif
    (void)h;
    return ((const R*)p)[i];
}
static void st(const orc* h, void* p, uint64_t i, R x) {
#ifdef ORC_PREC_F32
    if (h->ft == ION_FP16S) { ((uint16_t*)p)[i] = ieee_float_to_half_rne(x * 32768.0f); return; }
    if (h->ft == ION_FP16C) { ((uint16_t*)p)[i] = fp16c_encode(x); return; }
#endif
    (void)h;
    ((R*)p)[i] = x;
}

/* ------------------------------------------------------------------------
 * Units -> kernel constants: src/lbm/units.rs:149-197 (f32 arithmetic as in
 * Rust, f64 parts where the reference computes in f64), DEF_W
 * (src/lbm/domain.rs:808), DEF_KMU (839), DEF_WQ (848).
 * ---------------------------------------------------------------------- */
static float sqf(float x) { return x * x; }
static float cbf(float x) { return x * x * x; }
static float to4f(float x) { return x * x * x * x; }
static double atom_mass(int p) {
    switch (p) {
        case ION_PROP_HE: return 6.6464731e-27;
        case ION_PROP_NE: return 3.3509177e-26;
        case ION_PROP_AR: return 6.6335209e-26;
        case ION_PROP_KR: return 1.3914984e-25;
        case ION_PROP_XE: return 2.1801714e-25;
        default: return 1.6735575e-27;
    }
}
int orc_constants(const ion_config* c, ion_constants* k) {
    const ion_units* u = &c->units;
    const float pi = (float)3.14159265358979323846;
    memset(k, 0, sizeof(*k));
    k->w = 1.0f / (3.0f * c->nu + 0.5f);
    k->epsilon_0 = 8.8541878128E-12f / ((sqf(u->a) * to4f(u->s)) / (u->kg * cbf(u->m)));
    k->ke = 1.0f / (4.0f * pi * k->epsilon_0);
    k->mu_0 = 1.256637062E-6f / ((u->kg * u->m) / (sqf(u->a) * sqf(u->s)));
    k->kmu = k->mu_0 / (4.0f * pi);
    k->kmu0 = k->mu_0;
    k->kkge = (float)(9.1093837139E-31 / -1.602176634E-19) / (u->kg / (u->a * u->s));
    k->kimg = (float)((1.0 / (atom_mass(u->prop) * 1e20)) / (double)u->kg);
    k->kvev = (float)(9.1093837139E-31 / (2.0 * 1.602176634E-19) / (double)u->kg);
    k->kme = (float)(5.68563006E-12 / ((double)u->kg / ((double)u->a * (double)u->s)));
    k->wq = 1.0f / (2.0f * 1.0f + 0.5f); /* k_charge_expansion_lu() = 1 (units.rs:169-173) */
    /* SUBGRID_ECR: kkBme_lu, keabs_lu (units.rs:187-193), f64 arithmetic rounded to f32 */
    k->kkbme = (float)(-22734499.72063751808909449412 /
                       (((double)u->m * (double)u->m) / (((double)u->s * (double)u->s) * (double)u->k)));
    k->keabs = (float)(1.40897016100511360652E-8 /
                       ((((double)u->a * (double)u->a) * ((double)u->s * (double)u->s)) / (double)u->kg));
    return 0;
}

/* ------------------------------------------------------------------------
 * lattice geometry: index <-> coordinates (sim_kernels.cl:131-144),
 * periodic neighbours (248-302), D3Q7 neighbours (382-389)
 * ---------------------------------------------------------------------- */
static void coords(const orc* h, uint64_t n, uint32_t* x, uint32_t* y, uint32_t* z) {
    const uint64_t xy = (uint64_t)h->nx * h->ny, t = n % xy;
    *x = (uint32_t)(t % h->nx); *y = (uint32_t)(t / h->nx); *z = (uint32_t)(n / xy);
}
static uint32_t wrapc(int64_t v, uint32_t nmax) { return (uint32_t)((v + nmax) % nmax); }
static void neighbours(const orc* h, uint64_t n, uint64_t* j) {
    uint32_t x, y, z;
    coords(h, n, &x, &y, &z);
    for (int i = 0; i < h->vs->q; i++) {
        const signed char* c = h->vs->c[i];
        j[i] = wrapc((int64_t)x + c[0], h->nx) + ((uint64_t)wrapc((int64_t)y + c[1], h->ny) +
               (uint64_t)wrapc((int64_t)z + c[2], h->nz) * h->ny) * h->nx;
    }
}
static void neighbours7(const orc* h, uint64_t n, uint64_t* j) {
    static const signed char c7[7][3] = {{0,0,0},{1,0,0},{-1,0,0},{0,1,0},{0,-1,0},{0,0,1},{0,0,-1}};
    uint32_t x, y, z;
    coords(h, n, &x, &y, &z);
    for (int i = 0; i < 7; i++)
        j[i] = wrapc((int64_t)x + c7[i][0], h->nx) + ((uint64_t)wrapc((int64_t)y + c7[i][1], h->ny) +
               (uint64_t)wrapc((int64_t)z + c7[i][2], h->nz) * h->ny) * h->nx;
}

/* Esoteric-Pull in-place streaming: load_f / store_f (sim_kernels.cl:234-247),
 * load_a / store_a for the D3Q7 lattice (397-410). */
static void ep_load(const orc* h, const void* f, int q, uint64_t n, const uint64_t* j, uint64_t t, R* v) {
    const uint64_t N = h->n;
    v[0] = ld(h, f, n);
    for (int i = 1; i < q; i += 2) {
        v[i] = ld(h, f, (uint64_t)((t & 1u) ? i : i + 1) * N + n);
        v[i + 1] = ld(h, f, (uint64_t)((t & 1u) ? i + 1 : i) * N + j[i]);
    }
}
static void ep_store(const orc* h, void* f, int q, uint64_t n, const uint64_t* j, uint64_t t, const R* v) {
    const uint64_t N = h->n;
    st(h, f, n, v[0]);
    for (int i = 1; i < q; i += 2) {
        st(h, f, (uint64_t)((t & 1u) ? i + 1 : i) * N + j[i], v[i]);
        st(h, f, (uint64_t)((t & 1u) ? i : i + 1) * N + n, v[i + 1]);
    }
}

/* ------------------------------------------------------------------------
 * moments, equilibria, forcing
 * ---------------------------------------------------------------------- */
/* density and velocity from DDF-shifted populations (sim_kernels.cl:208-233):
 * rho sums f0..f(q-1) in order and adds 1 last; each velocity component is
 * the alternating sum over direction pairs, the positive member first. */
static void moments(const vset* vs, const R* f, R* rho, R* ux, R* uy, R* uz) {
    R r = f[0];
    for (int i = 1; i < vs->q; i++) r = r + f[i];
    r = r + (R)1;
    R u[3];
    for (int a = 0; a < 3; a++) {
        int first = 1;
        R acc = (R)0;
        for (int i = 1; i < vs->q; i += 2) {
            const int s = vs->c[i][a];
            if (!s) continue;
            const R pos = s > 0 ? f[i] : f[i + 1], neg = s > 0 ? f[i + 1] : f[i];
            acc = first ? pos - neg : (acc + pos) - neg;
            first = 0;
        }
        u[a] = first ? (R)0 : acc; /* D2Q9 leaves uz = 0 (sim_kernels.cl:215) */
    }
    *rho = r;
    if (vs->dims == 2) { *ux = u[0] / r; *uy = u[1] / r; *uz = (R)0 / r; }
    else { *ux = u[0] / r; *uy = u[1] / r; *uz = u[2] / r; }
}

/* c_i . v summed over the non-zero components in x, y, z order, the first
 * one carrying its sign (the u0..u9 pre-sums of sim_kernels.cl:162-205). */
static R project(const signed char* c, R vx, R vy, R vz) {
    const R comp[3] = {vx, vy, vz};
    int first = 1;
    R acc = (R)0;
    for (int a = 0; a < 3; a++) {
        if (!c[a]) continue;
        if (first) { acc = c[a] > 0 ? comp[a] : -comp[a]; first = 0; }
        else acc = c[a] > 0 ? acc + comp[a] : acc - comp[a];
    }
    return acc;
}

/* second-order equilibrium, DDF-shifted (sim_kernels.cl:155-207) */
static void equilibrium(const orc* h, R rho, R ux, R uy, R uz, R* feq) {
    const vset* vs = h->vs;
    const R c3 = (R)-3 * ((ux * ux + uy * uy) + uz * uz), rm1 = rho - (R)1;
    ux = ux * (R)3; uy = uy * (R)3; uz = uz * (R)3;
    feq[0] = h->wgt[0] * RFMA(rho, (R)0.5 * c3, rm1);
    for (int i = 1; i < vs->q; i += 2) {
        const R wr = h->wgt[vs->wc[i]] * rho, wrm1 = h->wgt[vs->wc[i]] * rm1;
        const R p = project(vs->c[i], ux, uy, uz);
        feq[i] = RFMA(wr, RFMA((R)0.5, RFMA(p, p, c3), p), wrm1);
        feq[i + 1] = RFMA(wr, RFMA((R)0.5, RFMA(p, p, c3), -p), wrm1);
    }
}

/* Guo forcing terms (sim_kernels.cl:367-377) */
static void forcing(const orc* h, R ux, R uy, R uz, R fx, R fy, R fz, R* Fin) {
    const vset* vs = h->vs;
    const R uF = vs->dims == 2 ? -(R)THIRD_F * RFMA(ux, fx, uy * fy) : -(R)THIRD_F * RFMA(ux, fx, RFMA(uy, fy, uz * fz));
    Fin[0] = ((R)9 * h->wgt[0]) * uF;
    for (int i = 1; i < vs->q; i++) {
        const R cx = vs->c[i][0], cy = vs->c[i][1], cz = vs->c[i][2];
        const R cf = (cx * fx + cy * fy) + cz * fz;
        const R cu = ((cx * ux + cy * uy) + cz * uz) + (R)THIRD_F;
        Fin[i] = ((R)9 * h->wgt[vs->wc[i]]) * RFMA(cf, cu, uF);
    }
}

/* D3Q7 advection equilibrium, DDF-shifted (sim_kernels.cl:390-396) */
static void adv_equilibrium(R Q, R ux, R uy, R uz, R* a) {
    const R hq = (R)0.5 * Q, eq = (R)0.125 * (Q - (R)1);
    a[0] = RFMA((R)0.25, Q, (R)-0.25);
    a[1] = RFMA(hq, ux, eq); a[2] = RFMA(hq, -ux, eq);
    a[3] = RFMA(hq, uy, eq); a[4] = RFMA(hq, -uy, eq);
    a[5] = RFMA(hq, uz, eq); a[6] = RFMA(hq, -uz, eq);
}

static R clampr(R x, R lo, R hi) { return RMIN(RMAX(x, lo), hi); }

/* LOD bin of a cell at depth d (sim_kernels.cl:425-433) */
static uint32_t lod_bin(const orc* h, uint64_t n, uint32_t d) {
    uint32_t x, y, z;
    coords(h, n, &x, &y, &z);
    const uint32_t nd = 1u << d;
    return x / (h->nx / nd) + (y / (h->ny / nd) + z / (h->nz / nd) * nd) * nd;
}

/* ------------------------------------------------------------------------
 * one cell of stream_collide (sim_kernels.cl:465-758)
 * ---------------------------------------------------------------------- */
/* SUBGRID_ECR block of stream_collide (sim_kernels.cl:557-629) with mag_v /
 * grad_mag_v (449-461): electron temperature on a D3Q7 lattice, ECR heating
 * by the part of E_var perpendicular to B, guiding-centre drift along
 * -grad|B| (the reference's a - b/2 difference), the placeholder ionisation
 * 1e-4 Et added to the electron and the gas charge. */
static R mag_v(const orc* h, const R* V, uint64_t m) {
    const uint64_t N = h->n;
    return RSQRT((V[m] * V[m] + V[N + m] * V[N + m]) + V[2 * N + m] * V[2 * N + m]);
}
static void ecr_cell(orc* h, uint64_t n, const uint64_t* j7, uint64_t t, R Bx, R By, R Bz, R* rhoe, R* rhoq, R* uxe,
                     R* uye, R* uze) {
    const uint64_t N = h->n;
    R ethn[7];
    ep_load(h, h->eti, 7, n, j7, t, ethn);
    R Etn = (R)0;
    for (int i = 0; i < 7; i++) Etn = Etn + ethn[i];
    Etn = Etn + (R)1;
    const R Evx = h->e_var[n], Evy = h->e_var[N + n], Evz = h->e_var[2 * N + n];
    const R lB = RSQRT((Bx * Bx + By * By) + Bz * Bz);
    const R kpar = ((Evx * Bx + Evy * By) + Evz * Bz) / (lB * lB);
    const R pex = Evx - kpar * Bx, pey = Evy - kpar * By, pez = Evz - kpar * Bz;
    const R Emag = RSQRT((pex * pex + pey * pey) + pez * pez);
    Etn = Etn + (((h->keabs / h->kkbme) * (*rhoe + (R)0.00001f)) / h->kkge) * (Emag * Emag);
    uint32_t x, y, z;
    coords(h, n, &x, &y, &z);
    R gx = (R)0, gy = (R)0, gz = (R)0;
    if (!(x == 0 || x == h->nx - 1 || y == 0 || y == h->ny - 1 || z == 0 || z == h->nz - 1)) {
        const uint64_t sy = h->nx, sz = (uint64_t)h->nx * h->ny;
        gx = mag_v(h, h->b_dyn, n + 1) - mag_v(h, h->b_dyn, n - 1) / (R)2;
        gy = mag_v(h, h->b_dyn, n + sy) - mag_v(h, h->b_dyn, n - sy) / (R)2;
        gz = mag_v(h, h->b_dyn, n + sz) - mag_v(h, h->b_dyn, n - sz) / (R)2;
    }
    const R kt = h->kkbme * Etn;
    const R dux = (kt * gx) / lB, duy = (kt * gy) / lB, duz = (kt * gz) / lB;
    *uxe = *uxe + dux; *uye = *uye + duy; *uze = *uze + duz;
    Etn = Etn - RSQRT((dux * dux + duy * duy) + duz * duz) / h->kkbme;
    R eteq[7];
    adv_equilibrium(Etn, *uxe, *uye, *uze, eteq);
    if (h->cfg.update_fields) h->et[n] = Etn;
    for (int i = 0; i < 7; i++) ethn[i] = RFMA((R)1 - h->wq, ethn[i], h->wq * eteq[i]);
    ep_store(h, h->eti, 7, n, j7, t, ethn);
    const R dq = (R)0.0001f * Etn;
    *rhoe = *rhoe + dq;
    *rhoq = *rhoq + dq;
}

static void collide_cell(orc* h, uint64_t n, uint64_t t) {
    const vset* vs = h->vs;
    const int q = vs->q;
    const ion_config* c = &h->cfg;
    const uint64_t N = h->n;
    const uint8_t fbo = h->flags[n] & F_BO;
    if (h->lodm) h->lodm[n] = 0;
    if (fbo == F_S) return;
    const int eq_cell = c->ext_equilibrium_boundaries && fbo == F_E;

    uint64_t j[19];
    neighbours(h, n, j);
    R fhn[19], feq[19], Fin[19];
    ep_load(h, h->fi, q, n, j, t, fhn);
    R rhon, uxn, uyn, uzn;
    if (eq_cell) { rhon = h->rho[n]; uxn = h->u[n]; uyn = h->u[N + n]; uzn = h->u[2 * N + n]; }
    else moments(vs, fhn, &rhon, &uxn, &uyn, &uzn);

    R fxn = c->f_x, fyn = c->f_y, fzn = c->f_z;
    const R w = h->w;
    const R c_tau = RFMA(w, (R)-0.5, (R)1);
    if (c->ext_force_field) { fxn = fxn + h->F[n]; fyn = fyn + h->F[N + n]; fzn = fzn + h->F[2 * N + n]; }

    if (c->ext_magneto_hydro) {
        /* cached fields (532-533) */
        const R Bx = h->b_dyn[n], By = h->b_dyn[N + n], Bz = h->b_dyn[2 * N + n];
        const R Ex = h->e_dyn[n], Ey = h->e_dyn[N + n], Ez = h->e_dyn[2 * N + n];
        /* electron gas, part 1 (537-540) */
        R ehn[19];
        ep_load(h, h->ei, q, n, j, t, ehn);
        R rhoe, uxe, uye, uze;
        moments(vs, ehn, &rhoe, &uxe, &uye, &uze);
        /* charge advection, part 1 (547-553) */
        uint64_t j7[7];
        neighbours7(h, n, j7);
        R qhn[7];
        ep_load(h, h->fqi, 7, n, j7, t, qhn);
        R rhoq = (R)0;
        for (int i = 0; i < 7; i++) rhoq = rhoq + qhn[i];
        rhoq = rhoq + (R)1;
        if (h->eti) ecr_cell(h, n, j7, t, Bx, By, Bz, &rhoe, &rhoq, &uxe, &uye, &uze);
        /* charge advection, part 2 (633-637) */
        h->qf[n] = rhoq - rhoe;
        R aeq[7];
        adv_equilibrium(rhoq, uxn, uyn, uzn, aeq);
        for (int i = 0; i < 7; i++) qhn[i] = RFMA((R)1 - h->wq, qhn[i], h->wq * aeq[i]);
        ep_store(h, h->fqi, 7, n, j7, t, qhn);
        /* electron gas, part 2 (641-656) */
        const R cxv = uye * Bz - uze * By, cyv = uze * Bx - uxe * Bz, czv = uxe * By - uye * Bx;
        const R nre = -rhoe;
        const R efx = nre * (Ex + cxv), efy = nre * (Ey + cyv), efz = nre * (Ez + czv);
        const R r2e = (R)0.5 / (rhoe * h->kkge);
        uxe = clampr(RFMA(efx, r2e, uxe), -(R)CS_F, (R)CS_F);
        uye = clampr(RFMA(efy, r2e, uye), -(R)CS_F, (R)CS_F);
        uze = clampr(RFMA(efz, r2e, uze), -(R)CS_F, (R)CS_F);
        forcing(h, uxe, uye, uze, efx, efy, efz, Fin);
        equilibrium(h, rhoe, uxe, uye, uze, feq);
        for (int i = 0; i < q; i++) Fin[i] = Fin[i] * c_tau;
        for (int i = 0; i < q; i++)
            ehn[i] = eq_cell ? feq[i] : RFMA((R)1 - w, ehn[i], RFMA(w, feq[i], Fin[i]));
        ep_store(h, h->ei, q, n, j, t, ehn);
        /* Lorentz force on the gas (660-662) */
        fxn = fxn + rhoq * ((Ex + uyn * Bz) - uzn * By);
        fyn = fyn + rhoq * ((Ey + uzn * Bx) - uxn * Bz);
        fzn = fzn + rhoq * ((Ez + uxn * By) - uyn * Bx);
        /* LOD contribution (666-677), summed later in cell order */
        if (h->depth > 0 && h->lodc) {
            const uint32_t nd = 1u << h->depth;
            const R ils = (R)1 / (R)((h->nx / nd) * (h->ny / nd) * (h->nz / nd));
            h->lodc[4 * n + 0] = rhoq - rhoe;
            h->lodc[4 * n + 1] = uxn * ils;
            h->lodc[4 * n + 2] = uyn * ils;
            h->lodc[4 * n + 3] = uzn * ils;
            h->lodm[n] = 1;
        }
    }

    if (c->ext_volume_force) { /* Guo half-step and forcing terms (680-685) */
        const R r2 = (R)0.5 / rhon;
        uxn = clampr(RFMA(fxn, r2, uxn), -(R)CS_F, (R)CS_F);
        uyn = clampr(RFMA(fyn, r2, uyn), -(R)CS_F, (R)CS_F);
        uzn = clampr(RFMA(fzn, r2, uzn), -(R)CS_F, (R)CS_F);
        forcing(h, uxn, uyn, uzn, fxn, fyn, fzn, Fin);
    } else { /* 686-690 */
        uxn = clampr(uxn, -(R)CS_F, (R)CS_F);
        uyn = clampr(uyn, -(R)CS_F, (R)CS_F);
        uzn = clampr(uzn, -(R)CS_F, (R)CS_F);
        for (int i = 0; i < q; i++) Fin[i] = (R)0;
    }
    if (c->update_fields && !eq_cell) { /* 694-710 */
        h->rho[n] = rhon; h->u[n] = uxn; h->u[N + n] = uyn; h->u[2 * N + n] = uzn;
    }
    equilibrium(h, rhon, uxn, uyn, uzn, feq);

    if (c->relaxation_time == ION_TRT) { /* 725-754 */
        const R wp = w, wm = (R)1 / ((R)0.1875 / ((R)1 / w - (R)0.5) + (R)0.5);
        if (c->ext_volume_force) {
            const R ctp = RFMA(wp, (R)-0.25, (R)0.5), ctm = RFMA(wm, (R)-0.25, (R)0.5);
            R Fb[19];
            Fb[0] = Fin[0];
            for (int i = 1; i < q; i += 2) { Fb[i] = Fin[i + 1]; Fb[i + 1] = Fin[i]; }
            for (int i = 0; i < q; i++) Fin[i] = RFMA(ctp, Fin[i] + Fb[i], ctm * (Fin[i] - Fb[i]));
        }
        R fb[19], eb[19];
        fb[0] = fhn[0]; eb[0] = feq[0];
        for (int i = 1; i < q; i += 2) { fb[i] = fhn[i + 1]; fb[i + 1] = fhn[i]; eb[i] = feq[i + 1]; eb[i + 1] = feq[i]; }
        for (int i = 0; i < q; i++) {
            const R sym = ((feq[i] - fhn[i]) + eb[i]) - fb[i];
            const R asym = ((feq[i] - eb[i]) - fhn[i]) + fb[i];
            fhn[i] = eq_cell ? feq[i] : RFMA((R)0.5 * wp, sym, RFMA((R)0.5 * wm, asym, fhn[i] + Fin[i]));
        }
    } else { /* SRT, 714-723 */
        if (c->ext_volume_force) for (int i = 0; i < q; i++) Fin[i] = Fin[i] * c_tau;
        for (int i = 0; i < q; i++) fhn[i] = eq_cell ? feq[i] : RFMA((R)1 - w, fhn[i], RFMA(w, feq[i], Fin[i]));
    }
    ep_store(h, h->fi, q, n, j, t, fhn);
}

/* ------------------------------------------------------------------------
 * update_e_b_dynamic for one cell (sim_kernels.cl:897-993), one domain:
 * near field over the cell's aligned block of max(N/2^(2^D),1) cells, then
 * the depth-D LOD bins [n_lod_own - 8^D, n_lod_own) except the cell's own.
 * ---------------------------------------------------------------------- */
static void add_source(R rx, R ry, R rz, R qc, R vx, R vy, R vz, R* e, R* b) {
    const R s = RSQRT((rx * rx + ry * ry) + rz * rz);
    const R c3 = (s * s) * s;
    const R px = rx / c3, py = ry / c3, pz = rz / c3;
    e[0] = e[0] + qc * px; e[1] = e[1] + qc * py; e[2] = e[2] + qc * pz;
    const R bx = vy * pz - vz * py, by = vz * px - vx * pz, bz = vx * py - vy * px;
    b[0] = b[0] + qc * bx; b[1] = b[1] + qc * by; b[2] = b[2] + qc * bz;
}
static void field_cell(orc* h, uint64_t n) {
    if ((h->flags[n] & F_BO) == F_S) return;
    const uint64_t N = h->n;
    uint32_t x, y, z;
    coords(h, n, &x, &y, &z);
    const R fx = (R)x, fy = (R)y, fz = (R)z;
    const uint32_t D = h->depth, nd = 1u << D;
    uint32_t bs[3] = {h->nx / (1u << nd), h->ny / (1u << nd), h->nz / (1u << nd)};
    for (int a = 0; a < 3; a++) if (bs[a] < 1u) bs[a] = 1u;
    const uint32_t x0 = (x / bs[0]) * bs[0], y0 = (y / bs[1]) * bs[1], z0 = (z / bs[2]) * bs[2];
    const uint32_t x1 = x0 + bs[0] < h->nx ? x0 + bs[0] : h->nx;
    const uint32_t y1 = y0 + bs[1] < h->ny ? y0 + bs[1] : h->ny;
    const uint32_t z1 = z0 + bs[2] < h->nz ? z0 + bs[2] : h->nz;
    R e[3] = {0, 0, 0}, b[3] = {0, 0, 0};
    for (uint32_t cx = x0; cx < x1; cx++)
        for (uint32_t cy = y0; cy < y1; cy++)
            for (uint32_t cz = z0; cz < z1; cz++) {
                const uint64_t nc = cx + ((uint64_t)cy + (uint64_t)cz * h->ny) * h->nx;
                if (nc == n) continue;
                const R qc = h->qf[nc];
                if (qc == (R)0) continue;
                add_source(fx - (R)cx, fy - (R)cy, fz - (R)cz, qc, h->u[nc], h->u[N + nc], h->u[2 * N + nc], e, b);
            }
    uint32_t nbins = 1;
    for (int a = 0; a < h->vs->dims; a++) nbins *= nd;
    const uint32_t own = lod_bin(h, n, D);
    const uint32_t first = h->n_lod_own > nbins ? h->n_lod_own - nbins : 0u;
    const R dsx = (R)(h->nx / nd), dsy = (R)(h->ny / nd), dsz = (R)(h->nz / nd);
    for (uint32_t d = first; d < h->n_lod_own; d++) {
        if (d == own) continue;
        const uint32_t tt = d % (nd * nd);
        const R lx = (R)(tt % nd) * dsx + (R)0.5 * dsx;
        const R ly = (R)(tt / nd) * dsy + (R)0.5 * dsy;
        const R lz = (R)(d / (nd * nd)) * dsz + (R)0.5 * dsz;
        const R* L = h->qu_lod + 4 * (uint64_t)d;
        add_source(fx - lx, fy - ly, fz - lz, L[0], L[1], L[2], L[3], e, b);
    }
    h->e_dyn[n] = h->e_stat[n] + h->ke * e[0];
    h->e_dyn[N + n] = h->e_stat[N + n] + h->ke * e[1];
    h->e_dyn[2 * N + n] = h->e_stat[2 * N + n] + h->ke * e[2];
    h->b_dyn[n] = h->b_stat[n] + h->kmu * b[0];
    h->b_dyn[N + n] = h->b_stat[N + n] + h->kmu * b[1];
    h->b_dyn[2 * N + n] = h->b_stat[2 * N + n] + h->kmu * b[2];
}

static void field_update(orc* h) {
    const long long N = (long long)h->n;
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 256) if (g_threads > 1)
    for (long long n = 0; n < N; n++) field_cell(h, (uint64_t)n);
}

/* ------------------------------------------------------------------------
 * API (same C symbols as the reference-kernel host program, oracle/ref_shim)
 * ---------------------------------------------------------------------- */
static void* xcalloc(size_t n, size_t s) { return n ? calloc(n, s) : NULL; }

void* orc_create(const ion_config* cfg, const ion_constants* kin) {
    if (cfg->d_x != 1 || cfg->d_y != 1 || cfg->d_z != 1) return NULL;
    const vset* vs = cfg->velocity_set == ION_D2Q9 ? &VS_D2Q9 : cfg->velocity_set == ION_D3Q15 ? &VS_D3Q15 :
                     cfg->velocity_set == ION_D3Q19 ? &VS_D3Q19 : NULL;
    if (!vs) return NULL;
    if (vs->dims == 2 && cfg->n_z != 1) return NULL;
    if (cfg->ext_magneto_hydro && !cfg->ext_volume_force) return NULL;
    if (cfg->mhd_lod_depth > 4) return NULL;
    if (cfg->ext_magneto_hydro && cfg->mhd_lod_depth > 0) {
        const uint32_t nd = 1u << cfg->mhd_lod_depth;
        if (cfg->n_x % nd || cfg->n_y % nd || (vs->dims == 3 && cfg->n_z % nd)) return NULL;
    }
    orc* h = (orc*)calloc(1, sizeof(orc));
    h->cfg = *cfg;
    h->vs = vs;
    h->nx = cfg->n_x; h->ny = cfg->n_y; h->nz = cfg->n_z;
    h->n = (uint64_t)h->nx * h->ny * h->nz;
    h->depth = cfg->mhd_lod_depth;
    uint32_t cnt = 1;
    for (uint32_t i = 0; i < h->depth; i++) {
        uint32_t p = 1;
        for (int d = 0; d < vs->dims; d++) p *= 1u << (i + 1);
        cnt += p;
    }
    h->n_lod_own = cnt;
    ion_constants k;
    if (kin) k = *kin; else orc_constants(cfg, &k);
#ifdef ORC_PREC_F32
    h->w = k.w; h->ke = k.ke; h->kmu = k.kmu; h->kmu0 = k.kmu0; h->kkge = k.kkge; h->wq = k.wq;
    h->kkbme = k.kkbme; h->keabs = k.keabs;
    if (vs == &VS_D2Q9) { h->wgt[0] = 1.0f / 2.25f; h->wgt[1] = 1.0f / 9.0f; h->wgt[2] = 1.0f / 36.0f; }
    else if (vs == &VS_D3Q15) { h->wgt[0] = 1.0f / 4.5f; h->wgt[1] = 1.0f / 9.0f; h->wgt[2] = 1.0f / 72.0f; }
    else { h->wgt[0] = 1.0f / 3.0f; h->wgt[1] = 1.0f / 18.0f; h->wgt[2] = 1.0f / 36.0f; }
    h->ft = cfg->float_type;
#else
    {   /* FP64 oracle: constants evaluated in double from the same inputs */
        const ion_units* u = &cfg->units;
        const double pi = 3.14159265358979323846;
        const double eps0 = 8.8541878128E-12 / (((double)u->a * u->a * u->s * u->s * u->s * u->s) /
                                                  ((double)u->kg * u->m * u->m * u->m));
        const double mu0 = 1.256637062E-6 / (((double)u->kg * u->m) / ((double)u->a * u->a * u->s * u->s));
        h->w = 1.0 / (3.0 * (double)cfg->nu + 0.5);
        h->ke = 1.0 / (4.0 * pi * eps0);
        h->kmu = mu0 / (4.0 * pi);
        h->kmu0 = mu0;
        h->kkge = (9.1093837139E-31 / -1.602176634E-19) / ((double)u->kg / ((double)u->a * u->s));
        h->wq = 1.0 / 2.5;
        h->kkbme = -22734499.72063751808909449412 / (((double)u->m * u->m) / (((double)u->s * u->s) * u->k));
        h->keabs = 1.40897016100511360652E-8 / ((((double)u->a * u->a) * ((double)u->s * u->s)) / u->kg);
        (void)k;
    }
    if (vs == &VS_D2Q9) { h->wgt[0] = 1.0 / 2.25; h->wgt[1] = 1.0 / 9.0; h->wgt[2] = 1.0 / 36.0; }
    else if (vs == &VS_D3Q15) { h->wgt[0] = 1.0 / 4.5; h->wgt[1] = 1.0 / 9.0; h->wgt[2] = 1.0 / 72.0; }
    else { h->wgt[0] = 1.0 / 3.0; h->wgt[1] = 1.0 / 18.0; h->wgt[2] = 1.0 / 36.0; }
    h->ft = ION_FP32;
#endif
    const uint64_t N = h->n;
    const size_t dsz = h->ft == ION_FP32 ? sizeof(R) : sizeof(uint16_t);
    h->fi = xcalloc(N * vs->q, dsz);
    h->rho = (R*)xcalloc(N, sizeof(R));
    for (uint64_t i = 0; i < N; i++) h->rho[i] = (R)1;
    h->u = (R*)xcalloc(3 * N, sizeof(R));
    h->flags = (uint8_t*)xcalloc(N, 1);
    if (cfg->ext_force_field) h->F = (R*)xcalloc(3 * N, sizeof(R));
    if (cfg->ext_magneto_hydro) {
        const uint64_t npsi = (uint64_t)(h->nx + 2) * (h->ny + 2) * (h->nz + 2);
        h->e_dyn_count = npsi > 3 * N ? npsi : 3 * N;
        h->e_stat = (R*)xcalloc(3 * N, sizeof(R));
        h->b_stat = (R*)xcalloc(3 * N, sizeof(R));
        h->e_dyn = (R*)xcalloc(h->e_dyn_count, sizeof(R));
        h->b_dyn = (R*)xcalloc(3 * N, sizeof(R));
        h->fqi = xcalloc(7 * N, dsz);
        h->ei = xcalloc(N * vs->q, dsz);
        h->qf = (R*)xcalloc(N, sizeof(R));
        h->qu_lod = (R*)xcalloc((size_t)h->n_lod_own * 4, sizeof(R));
        if (h->depth > 0) { h->lodc = (R*)xcalloc(4 * N, sizeof(R)); h->lodm = (uint8_t*)xcalloc(N, 1); }
        if (cfg->ext_subgrid_ecr) { /* domain.rs:200-211 */
            h->e_var = (R*)xcalloc(3 * N, sizeof(R));
            h->eti = xcalloc(7 * N, dsz);
            h->et = (R*)xcalloc(N, sizeof(R));
        }
    }
    return h;
}

void orc_destroy(void* p) {
    orc* h = (orc*)p;
    if (!h) return;
    free(h->fi); free(h->fqi); free(h->ei); free(h->rho); free(h->u); free(h->F); free(h->e_stat);
    free(h->b_stat); free(h->e_dyn); free(h->b_dyn); free(h->qf); free(h->qu_lod); free(h->flags);
    free(h->lodc); free(h->lodm); free(h->e_var); free(h->eti); free(h->et);
    free(h);
}

void* orc_field(void* p, int field, size_t* elem_bytes, size_t* count) {
    orc* h = (orc*)p;
    const uint64_t N = h->n;
    const size_t dsz = h->ft == ION_FP32 ? sizeof(R) : sizeof(uint16_t);
    void* ptr = NULL;
    size_t eb = sizeof(R), c = 0;
    const int mhd = h->cfg.ext_magneto_hydro;
    switch (field) {
        case ION_FIELD_FI: ptr = h->fi; eb = dsz; c = N * h->vs->q; break;
        case ION_FIELD_RHO: ptr = h->rho; c = N; break;
        case ION_FIELD_U: ptr = h->u; c = 3 * N; break;
        case ION_FIELD_FLAGS: ptr = h->flags; eb = 1; c = N; break;
        case ION_FIELD_F: ptr = h->F; c = h->F ? 3 * N : 0; break;
        case ION_FIELD_E_STAT: ptr = h->e_stat; c = mhd ? 3 * N : 0; break;
        case ION_FIELD_B_STAT: ptr = h->b_stat; c = mhd ? 3 * N : 0; break;
        case ION_FIELD_E_DYN: ptr = h->e_dyn; c = mhd ? h->e_dyn_count : 0; break;
        case ION_FIELD_B_DYN: ptr = h->b_dyn; c = mhd ? 3 * N : 0; break;
        case ION_FIELD_FQI: ptr = h->fqi; eb = dsz; c = mhd ? 7 * N : 0; break;
        case ION_FIELD_EI: ptr = h->ei; eb = dsz; c = mhd ? N * h->vs->q : 0; break;
        case ION_FIELD_Q: ptr = h->qf; c = mhd ? N : 0; break;
        case ION_FIELD_QU_LOD: ptr = h->qu_lod; c = mhd ? (size_t)h->n_lod_own * 4 : 0; break;
        case ION_FIELD_E_VAR: ptr = h->e_var; c = h->e_var ? 3 * N : 0; break;
        case ION_FIELD_ETI: ptr = h->eti; eb = dsz; c = h->eti ? 7 * N : 0; break;
        case ION_FIELD_ET: ptr = h->et; c = h->et ? N : 0; break;
        default: break;
    }
    if (elem_bytes) *elem_bytes = eb;
    if (count) *count = c;
    return c ? ptr : NULL;
}

uint64_t orc_time_step(void* p) { return ((orc*)p)->t; }

/* The finite-plasma start (no reference counterpart, applied by the next
 * initialize): the electron gas starts at density rho_e0 instead of 0
 * (sim_kernels.cl:823) and the charge lattice at Q + rho_e0 instead of Q
 * (sim_kernels.cl:818), so the net charge Q is unchanged.  With rho_e0 = 0
 * initialize is the reference's. */
void orc_set_electron_background(void* p, float rho_e0) { ((orc*)p)->rho_e0 = (R)rho_e0; }

/* initialize kernel (sim_kernels.cl:760-832) + Lbm::initialize (mod.rs:214-231) */
void orc_initialize(void* p) {
    orc* h = (orc*)p;
    const uint64_t N = h->n;
    const int q = h->vs->q, mhd = h->cfg.ext_magneto_hydro;
    h->t = 1;
    const long long NN = (long long)N;
#pragma omp parallel for num_threads(g_threads) schedule(static) if (g_threads > 1)
    for (long long ii = 0; ii < NN; ii++) {
        const uint64_t n = (uint64_t)ii;
        uint64_t j[19];
        neighbours(h, n, j);
        if ((h->flags[n] & F_BO) == F_S) { /* solid cells: zero velocity (and charge) */
            h->u[n] = (R)0; h->u[N + n] = (R)0; h->u[2 * N + n] = (R)0;
            if (mhd) h->qf[n] = (R)0;
        }
        R feq[19];
        equilibrium(h, h->rho[n], h->u[n], h->u[N + n], h->u[2 * N + n], feq);
        ep_store(h, h->fi, q, n, j, 1, feq);
        if (mhd) {
            R aeq[7];
            uint64_t j7[7];
            /* finite-plasma start: ions at Q + rho_e0, electrons at rho_e0 */
            const R rhoq0 = h->rho_e0 != (R)0 ? h->qf[n] + h->rho_e0 : h->qf[n];
            adv_equilibrium(rhoq0, h->u[n], h->u[N + n], h->u[2 * N + n], aeq);
            neighbours7(h, n, j7);
            ep_store(h, h->fqi, 7, n, j7, 1, aeq);
            for (int c = 0; c < 3; c++) { h->b_dyn[c * N + n] = h->b_stat[c * N + n]; h->e_dyn[c * N + n] = h->e_stat[c * N + n]; }
            equilibrium(h, h->rho_e0, h->u[n], h->u[N + n], h->u[2 * N + n], feq);
            ep_store(h, h->ei, q, n, j, 1, feq);
            if (h->eti) { /* electron temperature DDFs (827-831) */
                adv_equilibrium(h->et[n], h->u[n], h->u[N + n], h->u[2 * N + n], aeq);
                ep_store(h, h->eti, 7, n, j7, 1, aeq);
            }
        }
    }
    if (mhd) field_update(h);
    h->t = 0;
}

/* Lbm::do_time_step (mod.rs:250-272): clear LOD, stream_collide, LOD sums,
 * update_e_b_dynamic */
void orc_do_time_step(void* p) {
    orc* h = (orc*)p;
    const uint64_t N = h->n, t = h->t;
    const int mhd = h->cfg.ext_magneto_hydro;
    const long long NN = (long long)N;
#pragma omp parallel for num_threads(g_threads) schedule(static) if (g_threads > 1)
    for (long long n = 0; n < NN; n++) collide_cell(h, (uint64_t)n, t);
    if (mhd) {
        memset(h->qu_lod, 0, sizeof(R) * 4 * (size_t)h->n_lod_own);
        if (h->depth > 0) {
            for (uint64_t n = 0; n < N; n++) {
                if (!h->lodm[n]) continue;
                R* L = h->qu_lod + 4 * (uint64_t)lod_bin(h, n, h->depth);
                for (int c = 0; c < 4; c++) L[c] = L[c] + h->lodc[4 * n + c];
            }
        }
        field_update(h);
    }
    h->t = t + 1;
}

void orc_run(void* p, uint64_t steps) {
    for (uint64_t i = 0; i < steps; i++) orc_do_time_step(p);
}

/* update_fields kernel (sim_kernels.cl:834-859) */
void orc_update_fields(void* p) {
    orc* h = (orc*)p;
    const uint64_t N = h->n;
    const long long NN = (long long)N;
#pragma omp parallel for num_threads(g_threads) schedule(static) if (g_threads > 1)
    for (long long ii = 0; ii < NN; ii++) {
        const uint64_t n = (uint64_t)ii;
        if ((h->flags[n] & F_BO) == F_S) continue;
        uint64_t j[19];
        R f[19], rho, ux, uy, uz;
        neighbours(h, n, j);
        ep_load(h, h->fi, h->vs->q, n, j, h->t, f);
        moments(h->vs, f, &rho, &ux, &uy, &uz);
        h->rho[n] = rho;
        h->u[n] = clampr(ux, -(R)CS_F, (R)CS_F);
        h->u[N + n] = clampr(uy, -(R)CS_F, (R)CS_F);
        h->u[2 * N + n] = clampr(uz, -(R)CS_F, (R)CS_F);
    }
}

/* ------------------------------------------------------------------------
 * Voxelisation: host part src/mesh.rs:281-343, column kernel
 * sim_kernels.cl:1150-1231 (Moeller-Trumbore ray casting in both directions,
 * up to 64 forward hits kept as 16-bit distances, inside/outside parity with
 * the backward-hit error correction).  Geometry stays in float in both builds.
 * ---------------------------------------------------------------------- */
typedef struct { float x, y, z; } f3;
static f3 v3s(f3 a, f3 b) { f3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static f3 v3x(f3 a, f3 b) { f3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; return r; }
static float v3d(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static int iclamp(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

int orc_voxelize(void* p, const float* p0, const float* p1, const float* p2, uint32_t ntri,
                 const float* pmin, const float* pmax, int model_type, float v0, float v1, float v2) {
    orc* h = (orc*)p;
    const uint64_t N = h->n;
    const float x0 = pmin[0] - 2.0f, y0 = pmin[1] - 2.0f, z0 = pmin[2] - 2.0f;
    const float x1 = pmax[0] + 2.0f, y1 = pmax[1] + 2.0f, z1 = pmax[2] + 2.0f;
    const float a0 = (y1 - y0) * (z1 - z0), a1 = (z1 - z0) * (x1 - x0), a2 = (x1 - x0) * (y1 - y0);
    const int dir = (a0 < a1 && a0 < a2) ? 0 : (a1 < a2 ? 1 : 2);
    const uint64_t A = dir == 0 ? (uint64_t)h->ny * h->nz : dir == 1 ? (uint64_t)h->nx * h->nz : (uint64_t)h->nx * h->ny;
    uint8_t flag;
    switch (model_type) {
        case ION_MODEL_SOLID: flag = 0x01; break;
        case ION_MODEL_MAGNET: flag = 0x11; break;
        case ION_MODEL_CHARGED: flag = 0x09; break;
        case ION_MODEL_CHARGED_ECR: flag = 0x05; break;
        default: return -1;
    }
    float mx = 0.0f, my = 0.0f, mz = 0.0f;
    const ion_units* un = &h->cfg.units;
    if (model_type == ION_MODEL_MAGNET) { mx = v0 / (un->a / un->m); my = v1 / (un->a / un->m); mz = v2 / (un->a / un->m); }
    else if (model_type != ION_MODEL_SOLID) mx = v0 / (un->a * un->s);
    const int nx = (int)h->nx, ny = (int)h->ny, nz = (int)h->nz;
    const f3 rdir = {(float)(dir == 0), (float)(dir == 1), (float)(dir == 2)};
    const long long AA = (long long)A;
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 64) if (g_threads > 1)
    for (long long aa = 0; aa < AA; aa++) {
        const uint32_t a = (uint32_t)aa;
        uint32_t c[3];
        if (dir == 0) { c[0] = (uint32_t)iclamp((int)x0, 0, nx - 1); c[1] = a % h->ny; c[2] = a / h->ny; }
        else if (dir == 1) { c[0] = a / h->nz; c[1] = (uint32_t)iclamp((int)y0, 0, ny - 1); c[2] = a % h->nz; }
        else { c[0] = a % h->nx; c[1] = a / h->nx; c[2] = (uint32_t)iclamp((int)z0, 0, nz - 1); }
        /* ray origin: position() + offset (single domain: OX=OY=OZ=0) */
        const f3 org = {(((float)c[0] + 0.5f) - 0.5f * (float)nx) + (0.5f * (float)nx - 0.5f),
                        (((float)c[1] + 0.5f) - 0.5f * (float)ny) + (0.5f * (float)ny - 0.5f),
                        (((float)c[2] + 0.5f) - 0.5f * (float)nz) + (0.5f * (float)nz - 0.5f)};
        int outside;
        if (dir == 0) outside = org.y < y0 || org.z < z0 || org.y >= y1 || org.z >= z1;
        else if (dir == 1) outside = org.x < x0 || org.z < z0 || org.x >= x1 || org.z >= z1;
        else outside = org.x < x0 || org.y < y0 || org.x >= x1 || org.y >= y1;
        if (outside) continue;
        uint16_t dist[64] = {0};
        uint32_t hits = 0, back = 0;
        for (uint32_t i = 0; i < ntri; i++) {
            const f3 P0 = {p0[3 * i], p0[3 * i + 1], p0[3 * i + 2]};
            const f3 P1 = {p1[3 * i], p1[3 * i + 1], p1[3 * i + 2]};
            const f3 P2 = {p2[3 * i], p2[3 * i + 1], p2[3 * i + 2]};
            const f3 e1 = v3s(P1, P0), e2 = v3s(P2, P0), s0 = v3s(org, P0);
            const f3 pv = v3x(rdir, e2), qv = v3x(s0, e1);
            const float inv = 1.0f / v3d(e1, pv);
            const float su = inv * v3d(s0, pv), sv = inv * v3d(rdir, qv), sd = inv * v3d(e2, qv);
            if (su >= 0.0f && su < 1.0f && sv >= 0.0f && su + sv < 1.0f) {
                if (sd > 0.0f) {
                    if (hits < 64u && sd < 65536.0f) dist[hits] = (uint16_t)sd;
                    hits++;
                } else {
                    back++;
                }
            }
        }
        const uint32_t ns = hits < 64u ? hits : 64u; /* the reference sorts out of bounds beyond 64 */
        for (uint32_t i = 1; i < ns; i++) {          /* insertion sort, ascending */
            const uint16_t key = dist[i];
            int k = (int)i - 1;
            while (k >= 0 && dist[k] > key) { dist[k + 1] = dist[k]; k--; }
            dist[k + 1] = key;
        }
        int inside = (hits % 2u) && (back % 2u);
        uint32_t next = (hits % 2u) != (back % 2u);
        const uint32_t h0 = c[dir];
        const uint32_t hmax = dir == 0 ? (uint32_t)iclamp((int)x1, 0, nx) : dir == 1 ? (uint32_t)iclamp((int)y1, 0, ny)
                                                                                      : (uint32_t)iclamp((int)z1, 0, nz);
        const uint32_t last = hits - 1u < 63u ? hits - 1u : 63u;
        const uint32_t hmesh = h0 + (uint32_t)dist[last];
        for (uint32_t hh = h0; hh < hmax; hh++) {
            while (next < hits && hh > h0 + (uint32_t)dist[next < 63u ? next : 63u]) { inside = !inside; next++; }
            inside = inside && (next < hits && hh < hmesh);
            uint32_t cc[3] = {c[0], c[1], c[2]};
            cc[dir] = hh;
            const uint64_t n = cc[0] + ((uint64_t)cc[1] + (uint64_t)cc[2] * h->ny) * h->nx;
            if (inside) {
                h->flags[n] = (uint8_t)((h->flags[n] & ~F_BO) | flag);
                if (h->cfg.ext_magneto_hydro) {
                    if (flag & F_M) { h->b_dyn[n] = mx; h->b_dyn[N + n] = my; h->b_dyn[2 * N + n] = mz; }
                    else if ((flag & F_F) || (flag & F_C)) h->b_dyn[n] = mx;
                }
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------
 * Static magnet field: psi_from_mesh (sim_kernels.cl:1234-1251) over the
 * padded (nx+2)(ny+2)(nz+2) grid, stored in E_dyn; static_b_from_mesh
 * (1253-1276): B_stat += -mu0 grad(psi) by central differences, skipped for
 * cells with bit 0 set.  Magnet cells are visited in ascending index order.
 * ---------------------------------------------------------------------- */
void orc_precompute_b(void* p) {
    orc* h = (orc*)p;
    if (!h->cfg.ext_magneto_hydro) return;
    const uint64_t N = h->n;
    uint64_t nm = 0;
    for (uint64_t i = 0; i < N; i++) nm += (h->flags[i] & F_M) != 0;
    uint64_t* mag = (uint64_t*)malloc(sizeof(uint64_t) * (nm ? nm : 1));
    nm = 0;
    for (uint64_t i = 0; i < N; i++) if (h->flags[i] & F_M) mag[nm++] = i;
    const uint32_t l0 = h->nx + 2, l1 = h->ny + 2;
    const long long NP = (long long)l0 * l1 * (h->nz + 2);
    R* psi = h->e_dyn;
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 256) if (g_threads > 1)
    for (long long np = 0; np < NP; np++) {
        const uint64_t t = (uint64_t)np % ((uint64_t)l0 * l1);
        const R cx = (R)(t % l0), cy = (R)(t / l0), cz = (R)((uint64_t)np / ((uint64_t)l0 * l1));
        R acc = (R)0;
        for (uint64_t k = 0; k < nm; k++) {
            const uint64_t i = mag[k];
            uint32_t x, y, z;
            coords(h, i, &x, &y, &z);
            const R dx = cx - (R)(x + 1u), dy = cy - (R)(y + 1u), dz = cz - (R)(z + 1u);
            const R l = RSQRT((dx * dx + dy * dy) + dz * dz);
            if (!(l == (R)0)) {
                const R mx = h->b_dyn[i], my = h->b_dyn[i + N], mz = h->b_dyn[i + 2 * N];
                acc = acc + ((dx * mx + dy * my) + dz * mz) / ((l * l) * l);
            }
        }
        psi[np] = (R)((double)acc / (4.0 * 3.14159265358979323846));
    }
    free(mag);
    const long long NN = (long long)N;
#pragma omp parallel for num_threads(g_threads) schedule(static) if (g_threads > 1)
    for (long long ii = 0; ii < NN; ii++) {
        const uint64_t n = (uint64_t)ii;
        if ((h->flags[n] & F_S) == F_S) continue;
        uint32_t x, y, z;
        coords(h, n, &x, &y, &z);
        const uint64_t c = (x + 1u) + ((uint64_t)(y + 1u) + (uint64_t)(z + 1u) * l1) * l0;
        const uint64_t zo = (uint64_t)l0 * l1;
        const R gx = (psi[c + 1] - psi[c - 1]) / (R)2, gy = (psi[c + l0] - psi[c - l0]) / (R)2,
                gz = (psi[c + zo] - psi[c - zo]) / (R)2;
        const R m = -h->kmu0;
        h->b_stat[n] = h->b_stat[n] + m * gx;
        h->b_stat[N + n] = h->b_stat[N + n] + m * gy;
        h->b_stat[2 * N + n] = h->b_stat[2 * N + n] + m * gz;
    }
}

/* static_e_from_mesh (sim_kernels.cl:1278-1300): E_stat += k_e sum q r/|r|^3
 * over charged-solid cells (charge held in B_dyn.x by the voxeliser). */
static void static_e_into(orc* h, R* E);
void orc_precompute_e(void* p) {
    orc* h = (orc*)p;
    if (!h->cfg.ext_magneto_hydro) return;
    static_e_into(h, h->e_stat);
}
/* Lbm::precompute_E_ECR (mod.rs:319-331): the same kernel into E_var (domain.rs:569-578) */
void orc_precompute_e_ecr(void* p) {
    orc* h = (orc*)p;
    if (!h->e_var) return;
    static_e_into(h, h->e_var);
}
static void static_e_into(orc* h, R* E) {
    const uint64_t N = h->n;
    const long long NN = (long long)N;
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 256) if (g_threads > 1)
    for (long long ii = 0; ii < NN; ii++) {
        const uint64_t n = (uint64_t)ii;
        if ((h->flags[n] & F_S) == F_S) continue;
        uint32_t x, y, z;
        coords(h, n, &x, &y, &z);
        R ex = 0, ey = 0, ez = 0;
        for (uint64_t i = 0; i < N; i++) {
            if (!((h->flags[i] & F_F) || (h->flags[i] & F_C))) continue;
            uint32_t a, b, c;
            coords(h, i, &a, &b, &c);
            const R dx = (R)x - (R)a, dy = (R)y - (R)b, dz = (R)z - (R)c;
            const R l = RSQRT((dx * dx + dy * dy) + dz * dz);
            if (l == (R)0) continue;
            const R q = h->b_dyn[i], l3 = (l * l) * l;
            ex = ex + (dx * q) / l3; ey = ey + (dy * q) / l3; ez = ez + (dz * q) / l3;
        }
        E[n] = E[n] + ex * h->ke;
        E[N + n] = E[N + n] + ey * h->ke;
        E[2 * N + n] = E[2 * N + n] + ez * h->ke;
    }
}

/* codec entry points for the codec tests */
uint16_t orc_fp16c_encode(float x) { return fp16c_encode(x); }
float orc_fp16c_decode(uint16_t x) { return fp16c_decode(x); }
uint16_t orc_fp16s_encode(float x) { return ieee_float_to_half_rne(x * 32768.0f); }
float orc_fp16s_decode(uint16_t x) { return ieee_half_to_float(x) * 3.0517578E-5f; }

int orc_kind(void) {
#ifdef ORC_PREC_F32
    return 2; /* restated oracle, float */
#else
    return 3; /* restated oracle, double */
#endif
}
