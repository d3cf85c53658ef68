// ion_ref_host.cpp -- test infrastructure (oracle), not product code.
//
// Host program around the reference's own kernels (IonSolver
// src/kernels/sim_kernels.cl, compiled as C++ through ion_ref_compat.hpp).
// It restates, for one domain, the host orchestration of
//   Lbm::new / LbmDomain::new  (src/lbm/mod.rs:166-210, src/lbm/domain.rs:88-212)
//   Lbm::initialize            (src/lbm/mod.rs:214-231)
//   Lbm::do_time_step          (src/lbm/mod.rs:250-272)
//   voxelize_mesh_on_device    (src/mesh.rs:281-343)
//   precompute_B / precompute_E (src/lbm/mod.rs:284-314, src/lbm/domain.rs:551-567)
// and exposes it with the same orc_* C API as the restated oracle
// (oracle/ion_oracle.c), so tests drive both the same way.
//
// Work-items run in index order on one thread unless orc_set_threads(n>1)
// is called (then OpenMP; the LOD float atomics make that order-dependent,
// exactly as on a GPU).
#include <vector>
#include <cstdio>

#include "ion_ref_compat.hpp"
#include "ionsolver.h"

namespace ionref {
uint g_nx, g_ny, g_nz, g_ax, g_ay, g_az, g_num_lod, g_num_lod_own;
ulong g_n;
int g_ox, g_oy, g_oz;
float g_dox, g_doy, g_doz;
float g_w, g_ke, g_kmu, g_kmu0, g_kkge, g_kimg, g_kvev, g_kme, g_wq, g_kkbme, g_keabs;
thread_local uint64_t g_gid;
}  // namespace ionref

#include ION_REF_VARIANT

// OpenCL address-space and function qualifiers carry no meaning on the host;
// kernel printf output is compiled out.
#define __kernel
#define kernel
#define __global
#define global
#define printf(...) ((void)0)
namespace ionref {
#include "sim_kernels_body.inc"
}  // namespace ionref
#undef __kernel
#undef kernel
#undef __global
#undef global
#undef printf

using namespace ionref;

namespace {

int g_threads = 1;

template <class F>
void launch(uint64_t count, F&& f) {
    if (g_threads > 1) {
#pragma omp parallel for num_threads(g_threads) schedule(static)
        for (long long i = 0; i < (long long)count; i++) {
            g_gid = (uint64_t)i;
            f();
        }
    } else {
        for (uint64_t i = 0; i < count; i++) {
            g_gid = i;
            f();
        }
    }
}

struct RefLbm {
    ion_config cfg;
    ion_constants k;
    uint nx, ny, nz;
    ulong n;
    uint q;
    uint n_lod, n_lod_own;
    ulong t;
    std::vector<fpxx> fi, fqi, ei, eti;
    std::vector<float> rho, u, F, e_stat, b_stat, e_dyn, b_dyn, qf, qu_lod, e_var, et;
    std::vector<uchar> flags;
    std::vector<float> bbu;
};

void set_globals(const RefLbm* h) {
    g_nx = h->nx; g_ny = h->ny; g_nz = h->nz; g_n = h->n;
    g_ax = h->ny * h->nz; g_ay = h->nz * h->nx; g_az = h->nx * h->ny;
    g_ox = 0; g_oy = 0; g_oz = 0;  // single domain: o = x*n_x/d_x - (d_x>1) = 0 (domain.rs:101-103)
    g_dox = 0.0f; g_doy = 0.0f; g_doz = 0.0f;
    g_num_lod = h->n_lod; g_num_lod_own = h->n_lod_own;
    g_w = h->k.w; g_ke = h->k.ke; g_kmu = h->k.kmu; g_kmu0 = h->k.kmu0; g_kkge = h->k.kkge;
    g_kimg = h->k.kimg; g_kvev = h->k.kvev; g_kme = h->k.kme; g_wq = h->k.wq;
    g_kkbme = h->k.kkbme; g_keabs = h->k.keabs;
}

// Units::magnetization_si_lu / charge_si_lu, src/lbm/units.rs:130-133, 145-147
float magnetization_si_lu(const ion_units& u, float m) { return m / (u.a / u.m); }
float charge_si_lu(const ion_units& u, float q) { return q / (u.a * u.s); }

}  // namespace

extern "C" {

void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }

void* orc_create(const ion_config* cfg, const ion_constants* k) {
    RefLbm* h = new RefLbm();
    h->cfg = *cfg;
    h->k = *k;
    h->nx = cfg->n_x; h->ny = cfg->n_y; h->nz = cfg->n_z;
    h->n = (ulong)h->nx * h->ny * h->nz;
    h->q = DEF_VELOCITY_SET;
    // n_lod_own = 1 + sum_{i<depth} (2^(i+1))^dims (domain.rs:110-115); one domain -> n_lod = n_lod_own
    uint c = 1;
    for (uint i = 0; i < (uint)cfg->mhd_lod_depth; i++) {
        uint s = 1u << (i + 1);
        uint p = 1;
        for (uint d = 0; d < DEF_DIMENSIONS; d++) p *= s;
        c += p;
    }
    h->n_lod_own = c;
    h->n_lod = c;
    h->t = 0;
    const ulong n = h->n;
    // buffer allocation, domain.rs:151-211 (rho starts at 1, all else at 0)
    h->fi.assign(n * h->q, (fpxx)0);
    h->rho.assign(n, 1.0f);
    h->u.assign(3 * n, 0.0f);
    h->flags.assign(n, 0);
    h->bbu.assign(16, 0.0f);
    if (cfg->ext_force_field) h->F.assign(3 * n, 0.0f);
#ifdef MAGNETO_HYDRO
    h->e_stat.assign(3 * n, 0.0f);
    h->b_stat.assign(3 * n, 0.0f);
    // psi_from_mesh writes (nx+2)(ny+2)(nz+2) values into E_dyn (domain.rs:280);
    // keep room for them when that exceeds 3N (tiny grids).
    ulong npsi = (ulong)(h->nx + 2) * (h->ny + 2) * (h->nz + 2);
    h->e_dyn.assign(npsi > 3 * n ? npsi : 3 * n, 0.0f);
    h->b_dyn.assign(3 * n, 0.0f);
    h->fqi.assign(7 * n, (fpxx)0);
    h->ei.assign(n * h->q, (fpxx)0);
    h->qf.assign(n, 0.0f);
    h->qu_lod.assign((size_t)h->n_lod * 4, 0.0f);
#endif
#ifdef SUBGRID_ECR
    // domain.rs:200-211
    h->e_var.assign(3 * n, 0.0f);
    h->eti.assign(7 * n, (fpxx)0);
    h->et.assign(n, 0.0f);
#endif
    return h;
}

void orc_destroy(void* p) { delete (RefLbm*)p; }

void* orc_field(void* p, int field, size_t* elem_bytes, size_t* count) {
    RefLbm* h = (RefLbm*)p;
    void* ptr = nullptr;
    size_t eb = 4, cnt = 0;
    switch (field) {
        case ION_FIELD_FI: ptr = h->fi.data(); eb = sizeof(fpxx); cnt = h->fi.size(); break;
        case ION_FIELD_RHO: ptr = h->rho.data(); cnt = h->rho.size(); break;
        case ION_FIELD_U: ptr = h->u.data(); cnt = h->u.size(); break;
        case ION_FIELD_FLAGS: ptr = h->flags.data(); eb = 1; cnt = h->flags.size(); break;
        case ION_FIELD_F: ptr = h->F.data(); cnt = h->F.size(); break;
        case ION_FIELD_E_STAT: ptr = h->e_stat.data(); cnt = h->e_stat.size(); break;
        case ION_FIELD_B_STAT: ptr = h->b_stat.data(); cnt = h->b_stat.size(); break;
        case ION_FIELD_E_DYN: ptr = h->e_dyn.data(); cnt = h->e_dyn.size(); break;
        case ION_FIELD_B_DYN: ptr = h->b_dyn.data(); cnt = h->b_dyn.size(); break;
        case ION_FIELD_FQI: ptr = h->fqi.data(); eb = sizeof(fpxx); cnt = h->fqi.size(); break;
        case ION_FIELD_EI: ptr = h->ei.data(); eb = sizeof(fpxx); cnt = h->ei.size(); break;
        case ION_FIELD_Q: ptr = h->qf.data(); cnt = h->qf.size(); break;
        case ION_FIELD_QU_LOD: ptr = h->qu_lod.data(); cnt = h->qu_lod.size(); break;
        case ION_FIELD_E_VAR: ptr = h->e_var.data(); cnt = h->e_var.size(); break;
        case ION_FIELD_ETI: ptr = h->eti.data(); eb = sizeof(fpxx); cnt = h->eti.size(); break;
        case ION_FIELD_ET: ptr = h->et.data(); cnt = h->et.size(); break;
        default: break;
    }
    if (elem_bytes) *elem_bytes = eb;
    if (count) *count = cnt;
    return cnt ? ptr : nullptr;
}

uint64_t orc_time_step(void* p) { return ((RefLbm*)p)->t; }

static void kernel_update_e_b(RefLbm* h) {
#ifdef MAGNETO_HYDRO
    launch(h->n, [&] {
        update_e_b_dynamic(h->e_stat.data(), h->b_stat.data(), h->e_dyn.data(), h->b_dyn.data(),
                           h->qf.data(), h->u.data(), h->qu_lod.data(), h->flags.data());
    });
#else
    (void)h;
#endif
}

// Lbm::initialize, src/lbm/mod.rs:214-231 (communicate_* are no-ops with one domain)
void orc_initialize(void* p) {
    RefLbm* h = (RefLbm*)p;
    set_globals(h);
    h->t += 1;
    launch(h->n, [&] {
        initialize(h->fi.data(), h->rho.data(), h->u.data(), h->flags.data()
#ifdef MAGNETO_HYDRO
                   , h->e_stat.data(), h->b_stat.data(), h->e_dyn.data(), h->b_dyn.data(),
                   h->fqi.data(), h->ei.data(), h->qf.data()
#endif
#ifdef SUBGRID_ECR
                   , h->eti.data(), h->et.data()
#endif
        );
    });
#ifdef MAGNETO_HYDRO
    kernel_update_e_b(h);
#endif
    h->t = 0;
}

// Lbm::do_time_step, src/lbm/mod.rs:250-272
void orc_do_time_step(void* p) {
    RefLbm* h = (RefLbm*)p;
    set_globals(h);
#ifdef MAGNETO_HYDRO
    launch(h->n_lod, [&] { clear_qu_lod(h->qu_lod.data()); });
#endif
    const ulong t = h->t;
    const float fx = h->cfg.f_x, fy = h->cfg.f_y, fz = h->cfg.f_z;
    launch(h->n, [&] {
        stream_collide(h->fi.data(), h->rho.data(), h->u.data(), h->flags.data(), t, fx, fy, fz
#ifdef FORCE_FIELD
                       , h->F.data()
#endif
#ifdef MAGNETO_HYDRO
                       , h->e_dyn.data(), h->b_dyn.data(), h->fqi.data(), h->ei.data(), h->qf.data(),
                       h->qu_lod.data()
#endif
#ifdef SUBGRID_ECR
                       , h->e_var.data(), h->eti.data(), h->et.data(), h->cfg.ecr_freq
#endif
        );
    });
#ifdef MAGNETO_HYDRO
    kernel_update_e_b(h);
#endif
    h->t += 1;
}

void orc_run(void* p, uint64_t steps) {
    for (uint64_t i = 0; i < steps; i++) orc_do_time_step(p);
}

// LbmDomain::enqueue_update_fields, src/lbm/domain.rs:432-441
void orc_update_fields(void* p) {
    RefLbm* h = (RefLbm*)p;
    set_globals(h);
    const ulong t = h->t;
    launch(h->n, [&] {
        update_fields(h->fi.data(), h->rho.data(), h->u.data(), h->flags.data(), t, h->cfg.f_x, h->cfg.f_y,
                      h->cfg.f_z);
    });
}

// LbmDomain::voxelize_mesh_on_device, src/mesh.rs:281-343
int orc_voxelize(void* p, const float* p0, const float* p1, const float* p2, uint32_t ntri,
                 const float* pmin, const float* pmax, int model_type, float v0, float v1, float v2) {
    RefLbm* h = (RefLbm*)p;
    set_globals(h);
    const float x0 = pmin[0] - 2.0f, y0 = pmin[1] - 2.0f, z0 = pmin[2] - 2.0f;
    const float x1 = pmax[0] + 2.0f, y1 = pmax[1] + 2.0f, z1 = pmax[2] + 2.0f;
    h->bbu.assign(16, 0.0f);
    h->bbu[0] = as_float(ntri);
    h->bbu[1] = x0; h->bbu[2] = y0; h->bbu[3] = z0; h->bbu[4] = x1; h->bbu[5] = y1; h->bbu[6] = z1;
    const float c0 = (y1 - y0) * (z1 - z0), c1 = (z1 - z0) * (x1 - x0), c2 = (x1 - x0) * (y1 - y0);
    const uint direction = (c0 < c1 && c0 < c2) ? 0u : (c1 < c2 ? 1u : 2u);
    const uint a[3] = {h->ny * h->nz, h->nx * h->nz, h->nx * h->ny};
    uchar flag = 0x01;
    float mx = 0.0f, my = 0.0f, mz = 0.0f;
    switch (model_type) {
        case ION_MODEL_SOLID: flag = 0x01; break;
        case ION_MODEL_MAGNET: flag = 0x11; break;
        case ION_MODEL_CHARGED: flag = 0x09; break;
        case ION_MODEL_CHARGED_ECR: flag = 0x05; break;
        default: return -1;
    }
    if (h->cfg.ext_magneto_hydro) {
        if (model_type == ION_MODEL_MAGNET) {
            mx = magnetization_si_lu(h->cfg.units, v0);
            my = magnetization_si_lu(h->cfg.units, v1);
            mz = magnetization_si_lu(h->cfg.units, v2);
        } else if (model_type == ION_MODEL_CHARGED || model_type == ION_MODEL_CHARGED_ECR) {
            mx = charge_si_lu(h->cfg.units, v0);
        }
    }
    const ulong t1 = h->t + 1;
    launch(a[direction], [&] {
        voxelize_mesh(direction, h->fi.data(), h->rho.data(), h->u.data(), h->flags.data(), t1, flag, p0, p1, p2,
                      h->bbu.data()
#ifdef MAGNETO_HYDRO
                      , mx, my, mz, h->b_dyn.data()
#endif
        );
    });
    (void)mx; (void)my; (void)mz;
    return 0;
}

// LbmDomain::enqueue_precompute_b, src/lbm/domain.rs:551-556
void orc_precompute_b(void* p) {
#ifdef MAGNETO_HYDRO
    RefLbm* h = (RefLbm*)p;
    set_globals(h);
    const ulong npsi = (ulong)(h->nx + 2) * (h->ny + 2) * (h->nz + 2);
    launch(npsi, [&] { psi_from_mesh(h->flags.data(), h->e_dyn.data(), h->b_dyn.data()); });
    launch(h->n, [&] { static_b_from_mesh(h->flags.data(), h->b_stat.data(), h->e_dyn.data()); });
#else
    (void)p;
#endif
}

// LbmDomain::enqueue_precompute_e, src/lbm/domain.rs:558-567
void orc_precompute_e(void* p) {
#ifdef MAGNETO_HYDRO
    RefLbm* h = (RefLbm*)p;
    set_globals(h);
    launch(h->n, [&] { static_e_from_mesh(h->flags.data(), h->e_stat.data(), h->b_dyn.data()); });
#else
    (void)p;
#endif
}

// LbmDomain::enqueue_precompute_e_ecr, src/lbm/domain.rs:569-578
void orc_precompute_e_ecr(void* p) {
#ifdef SUBGRID_ECR
    RefLbm* h = (RefLbm*)p;
    set_globals(h);
    launch(h->n, [&] { static_e_from_mesh(h->flags.data(), h->e_var.data(), h->b_dyn.data()); });
#else
    (void)p;
#endif
}

int orc_kind(void) { return 1; }  // 1 = the reference's kernels

// the reference's FP16C codec functions (sim_kernels.cl:79-90) and the
// FP16S load/store macros of get_device_defines (domain.rs:773-776)
uint16_t orc_fp16c_encode(float x) { return float_to_half_custom(x); }
float orc_fp16c_decode(uint16_t x) { return half_to_float_custom(x); }
uint16_t orc_fp16s_encode(float x) { half h[1]; vstore_half_rte((x) * 32768.0f, 0, h); return h[0]; }
float orc_fp16s_decode(uint16_t x) { const half h[1] = {x}; return vload_half(0, h) * 3.0517578E-5f; }

}  // extern "C"
