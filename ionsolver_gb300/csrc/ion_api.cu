// ion_api.cu -- the C ABI of include/ionsolver.h: a one-domain Lbm on one GPU.
//
// Host orchestration restated from IonSolver's Rust host
// (src/lbm/mod.rs, src/lbm/domain.rs, src/mesh.rs, src/file.rs,
// src/lbm/units.rs); kernels in lbm_q*.cu, field_kernels.cu,
// setup_kernels.cu.  Nothing here computes physics on the CPU.
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <thread>
#include <vector>

#include <memory>

#include "ion_device.cuh"
#include "ion_launch.h"
#include "surrogate.h"

using namespace ion;

namespace {

thread_local std::string g_error;
std::atomic<uint64_t> g_launches{0};

int fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_error = buf;
    return code;
}

#define CK(call)                                                                                      \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return fail(ION_E_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                           __FILE__, __LINE__);                                       \
    } while (0)

#define CKL()                                                                                         \
    do {                                                                                              \
        cudaError_t e_ = cudaGetLastError();                                                          \
        if (e_ != cudaSuccess) return fail(ION_E_CUDA, "kernel launch: %s (%s:%d)", cudaGetErrorString(e_), \
                                           __FILE__, __LINE__);                                       \
    } while (0)

}  // namespace

namespace ion {
int api_fail(int code, const char* message) { return fail(code, "%s", message); }
void api_count_launches(uint64_t n) { g_launches += n; }
}  // namespace ion

namespace {

// ---------------------------------------------------------------------------
// Units -> kernel constants (src/lbm/units.rs:149-197; domain.rs:808, 839, 848),
// evaluated in the same f32/f64 steps as the Rust code.
// ---------------------------------------------------------------------------
float sqf(float x) { return x * x; }
float cbf(float x) { return x * x * x; }
float to4f(float x) { return x * x * x * x; }
double atom_mass(int p) {
    switch (p) {
        case ION_PROP_HE: return 6.6464731e-27;
        case ION_PROP_NE: return 3.3509177e-26;
        case ION_PROP_AR: return 6.6335209e-26;
        case ION_PROP_KR: return 1.3914984e-25;
        case ION_PROP_XE: return 2.1801714e-25;
        default: return 1.6735575e-27;
    }
}
void derive_constants(const ion_config& c, ion_constants& k) {
    const ion_units& u = c.units;
    const float pi = (float)3.14159265358979323846;
    memset(&k, 0, sizeof k);
    k.w = 1.0f / (3.0f * c.nu + 0.5f);
    k.epsilon_0 = 8.8541878128E-12f / ((sqf(u.a) * to4f(u.s)) / (u.kg * cbf(u.m)));
    k.ke = 1.0f / (4.0f * pi * k.epsilon_0);
    k.mu_0 = 1.256637062E-6f / ((u.kg * u.m) / (sqf(u.a) * sqf(u.s)));
    k.kmu = k.mu_0 / (4.0f * pi);
    k.kmu0 = k.mu_0;
    k.kkge = (float)(9.1093837139E-31 / -1.602176634E-19) / (u.kg / (u.a * u.s));
    k.kimg = (float)((1.0 / (atom_mass(u.prop) * 1e20)) / (double)u.kg);
    k.kvev = (float)(9.1093837139E-31 / (2.0 * 1.602176634E-19) / (double)u.kg);
    k.kme = (float)(5.68563006E-12 / ((double)u.kg / ((double)u.a * (double)u.s)));
    k.wq = 1.0f / (2.0f * 1.0f + 0.5f);
    // SUBGRID_ECR (units.rs:187-193)
    k.kkbme = (float)(-22734499.72063751808909449412 /
                      (((double)u.m * (double)u.m) / (((double)u.s * (double)u.s) * (double)u.k)));
    k.keabs = (float)(1.40897016100511360652E-8 /
                      ((((double)u.a * (double)u.a) * ((double)u.s * (double)u.s)) / (double)u.kg));
}

int velocity_q(int vs) { return vs == ION_D2Q9 ? 9 : vs == ION_D3Q15 ? 15 : vs == ION_D3Q19 ? 19 : 27; }

int validate(const ion_config& c) {
    if (c.d_x != 1 || c.d_y != 1 || c.d_z != 1)
        return fail(ION_E_CONFIG, "d_x, d_y, d_z must be 1: this build runs one domain on one GPU");
    if (c.velocity_set == ION_D3Q27)
        return fail(ION_E_CONFIG, "D3Q27: the reference defines no DEF_WC for it (domain.rs:766-768), so it does not build");
    if (c.velocity_set < ION_D2Q9 || c.velocity_set > ION_D3Q19) return fail(ION_E_CONFIG, "unknown velocity_set %d", c.velocity_set);
    if (c.relaxation_time != ION_SRT && c.relaxation_time != ION_TRT) return fail(ION_E_CONFIG, "unknown relaxation_time");
    if (c.float_type < ION_FP16S || c.float_type > ION_FP32) return fail(ION_E_CONFIG, "unknown float_type");
    if (c.n_x == 0 || c.n_y == 0 || c.n_z == 0) return fail(ION_E_CONFIG, "grid sizes must be >= 1");
    // n_x * n_y fits in 64 bits; checked before the third factor so the product cannot wrap
    const uint64_t nxy = (uint64_t)c.n_x * c.n_y;
    if (nxy >= (1ull << 32) || nxy * c.n_z >= (1ull << 32))
        return fail(ION_E_CONFIG, "more than 2^32-1 cells (the reference indexes cells with uint)");
    if (c.velocity_set == ION_D2Q9 && c.n_z != 1) return fail(ION_E_CONFIG, "D2Q9 needs n_z == 1");
    if (c.ext_subgrid_ecr && !c.ext_magneto_hydro)
        return fail(ION_E_CONFIG, "ext_subgrid_ecr needs ext_magneto_hydro (as in the reference, mod.rs:79-80)");
    if (c.ext_magneto_hydro) {
        if (!c.ext_volume_force) return fail(ION_E_CONFIG, "ext_magneto_hydro needs ext_volume_force (as in the reference)");
        if (c.velocity_set == ION_D2Q9)
            return fail(ION_E_CONFIG, "ext_magneto_hydro needs a 3D velocity set (the reference divides by n_z/2^D = 0)");
        if (c.mhd_lod_depth > 4) return fail(ION_E_CONFIG, "mhd_lod_depth > 4 is not supported");
        const uint32_t nd = 1u << c.mhd_lod_depth;
        if (c.n_x % nd || c.n_y % nd || c.n_z % nd)
            return fail(ION_E_CONFIG, "with ext_magneto_hydro, n_x/n_y/n_z must be multiples of 2^mhd_lod_depth");
        if (c.field_mode > ION_FIELD_SURROGATE)
            return fail(ION_E_CONFIG, "field_mode %d is not available", (int)c.field_mode);
        if (c.field_mode == ION_FIELD_SURROGATE) {
            const uint32_t big = 1u << (1u << c.mhd_lod_depth);
            if (c.mhd_lod_depth < 2 || c.n_x / big > 1 || c.n_y / big > 1 || c.n_z / big > 1)
                return fail(ION_E_CONFIG, "the learned far field needs LOD depth >= 2 and an empty reference near field "
                                          "(n/2^(2^D) <= 1 on every axis)");
        }
    }
    if (c.ext_force_field && !c.ext_volume_force) return fail(ION_E_CONFIG, "ext_force_field needs ext_volume_force");
    return ION_OK;
}

__global__ void k_fill(float* p, uint64_t n, float v) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

struct HostMesh {
    std::vector<float> p0, p1, p2;  // [ntri][3]
    uint32_t ntri = 0;
    float pmin[3] = {0, 0, 0}, pmax[3] = {0, 0, 0}, center[3] = {0, 0, 0};
    // Mesh::update_bounds, src/mesh.rs:94-109
    void update_bounds() {
        if (!ntri) return;
        for (int a = 0; a < 3; a++) pmin[a] = pmax[a] = p0[a];
        for (uint32_t i = 0; i < ntri; i++)
            for (int a = 0; a < 3; a++) {
                const float x0 = p0[3 * i + a], x1 = p1[3 * i + a], x2 = p2[3 * i + a];
                pmin[a] = std::fmin(pmin[a], std::fmin(x2, std::fmin(x1, x0)));
                pmax[a] = std::fmax(pmax[a], std::fmax(x2, std::fmax(x1, x0)));
            }
    }
};

struct KEv {
    int kernel;
    cudaEvent_t a, b;
};

}  // namespace

struct ion_lbm {
    ion_config cfg{};
    ion_constants k{};
    DevLbm L{};
    cudaStream_t stream = nullptr;
    int q = 19;
    uint64_t t = 0;
    bool initialized = false;
    size_t e_dyn_count = 0;
    uint32_t* d_err = nullptr;
    double* d_partials = nullptr;
    double* d_sums = nullptr;
    uint32_t nparts = 0;
    uint32_t* d_tiles = nullptr;
    uint32_t* d_list = nullptr;
    uint32_t* d_count = nullptr;
    float *d_p0 = nullptr, *d_p1 = nullptr, *d_p2 = nullptr;
    size_t tri_cap = 0;
    std::vector<HostMesh> meshes;
    cudaGraphExec_t graph = nullptr;
    uint32_t graph_kernels = 0;
    bool graph_dirty = false;  // the step's launch sequence changed since capture
    cudaEvent_t ev[8] = {};
    bool ktiming = false;
    std::vector<KEv> kev;
    std::vector<cudaEvent_t> ev_pool;
    double ktime[3] = {0, 0, 0};
    uint64_t kcount[3] = {0, 0, 0};
    std::vector<void*> allocs;
    std::unique_ptr<ion::Surrogate> sur;  // learned far field (field_mode SURROGATE)
};

namespace {

int dmalloc(ion_lbm* h, void** p, size_t bytes) {
    *p = nullptr;
    if (!bytes) return ION_OK;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ION_E_NOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    }
    h->allocs.push_back(*p);
    return cudaMemsetAsync(*p, 0, bytes, h->stream) == cudaSuccess ? ION_OK : fail(ION_E_CUDA, "cudaMemsetAsync");
}

size_t ddf_bytes(int ft) { return ft == ION_FP32 ? 4 : 2; }

void destroy_handle(ion_lbm* h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    for (void* p : h->allocs) cudaFree(p);
    for (auto& e : h->ev) if (e) cudaEventDestroy(e);
    for (auto& e : h->kev) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
    for (auto e : h->ev_pool) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

// -------- launches of one step ---------------------------------------------
// kernel variant: 0 plain, 1 MAGNETO_HYDRO, 2 MAGNETO_HYDRO + SUBGRID_ECR
int lbm_mode(const ion_config& c) { return c.ext_magneto_hydro ? (c.ext_subgrid_ecr ? 2 : 1) : 0; }

int launch_stream_collide(ion_lbm* h, uint64_t t) {
    const int ft = h->cfg.float_type, mode = lbm_mode(h->cfg);
    const bool trt = h->cfg.relaxation_time == ION_TRT;
    if (h->q == 19) q19_stream_collide(h->L, ft, mode, trt, t, h->d_err, h->stream);
    else if (h->q == 15) q15_stream_collide(h->L, ft, mode, trt, t, h->d_err, h->stream);
    else q9_stream_collide(h->L, ft, mode, trt, t, h->d_err, h->stream);
    g_launches++;
    CKL();
    return ION_OK;
}

int launch_field(ion_lbm* h) {
    // the exact sum; SURROGATE handles use its FAST arithmetic outside the surrogate path
    launch_update_e_b(h->L, h->cfg.field_mode != ION_FIELD_BITWISE, h->d_err, h->stream);
    g_launches++;
    CKL();
    return ION_OK;
}

// learned far field + sampled exact check + device-decided exact fallback
int launch_surrogate_field(ion_lbm* h) {
    if (!h->sur || !h->sur->ready())
        return fail(ION_E_STATE, "field_mode SURROGATE: train (ion_lbm_surrogate_train) or load the network first");
    h->sur->step(h->L, h->stream, 0x2545F491u);
    launch_update_e_b_gated(h->L, h->d_err, h->sur->fallback_flag(), h->stream);
    g_launches += h->sur->launches_per_step() + 1;
    CKL();
    return ION_OK;
}

int launch_bins(ion_lbm* h) {
    if (h->L.depth > 0) {
        launch_lod_bins(h->L, h->stream);
        g_launches++;
        CKL();
    } else {
        CK(cudaMemsetAsync(h->L.qu_lod, 0, sizeof(float) * 4 * (size_t)h->L.n_lod_own, h->stream));
    }
    return ION_OK;
}

cudaEvent_t pool_event(ion_lbm* h) {
    if (!h->ev_pool.empty()) { cudaEvent_t e = h->ev_pool.back(); h->ev_pool.pop_back(); return e; }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

template <class F>
int timed(ion_lbm* h, int kernel, F&& f) {
    if (!h->ktiming) return f();
    KEv r{kernel, pool_event(h), pool_event(h)};
    cudaEventRecord(r.a, h->stream);
    const int rc = f();
    cudaEventRecord(r.b, h->stream);
    h->kev.push_back(r);
    return rc;
}

// Lbm::do_time_step (src/lbm/mod.rs:250-272) for step t
int enqueue_step(ion_lbm* h, uint64_t t) {
    int rc = timed(h, 0, [&] { return launch_stream_collide(h, t); });
    if (rc) return rc;
    if (h->cfg.ext_magneto_hydro) {
        rc = timed(h, 2, [&] { return launch_bins(h); });
        if (rc) return rc;
        rc = timed(h, 1, [&] {
            return h->cfg.field_mode == ION_FIELD_SURROGATE ? launch_surrogate_field(h) : launch_field(h);
        });
        if (rc) return rc;
    }
    return ION_OK;
}

uint32_t kernels_per_step(const ion_lbm* h) {
    uint32_t k = 1u + (h->cfg.ext_magneto_hydro ? (h->L.depth > 0 ? 2u : 1u) : 0u);
    if (h->cfg.ext_magneto_hydro && h->cfg.field_mode == ION_FIELD_SURROGATE && h->sur) k += h->sur->launches_per_step();
    return k;
}

int check_device_error(ion_lbm* h) {
    uint32_t err = 0;
    CK(cudaMemcpyAsync(&err, h->d_err, 4, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (err) {
        CK(cudaMemsetAsync(h->d_err, 0, 4, h->stream));
        return fail(ION_E_TIMEOUT, "a field-kernel shared-memory tile did not arrive within its wait limit");
    }
    return ION_OK;
}

// -------- STL (Mesh::read_stl_raw, src/mesh.rs:175-220) --------------------
struct Mat3 { float xx, xy, xz, yx, yy, yz, zx, zy, zz; };
Mat3 rot_around(float vx, float vy, float vz, float r) {  // src/mesh.rs:57-66
    const float sr = std::sin(r), cr = std::cos(r);
    auto sq = [](float x) { return x * x; };
    Mat3 m;
    m.xx = sq(vx) + (1.0f - sq(vx)) * cr; m.xy = vx * vy * (1.0f - cr) - vz * sr; m.xz = vx * vz * (1.0f - cr) + vy * sr;
    m.yx = vx * vy * (1.0f - cr) + vz * sr; m.yy = sq(vy) + (1.0f - sq(vy)) * cr; m.yz = vy * vz * (1.0f - cr) - vx * sr;
    m.zx = vx * vz * (1.0f - cr) - vy * sr; m.zy = vy * vz * (1.0f - cr) + vx * sr; m.zz = sq(vz) + (1.0f - sq(vz)) * cr;
    return m;
}
Mat3 matmul(const Mat3& a, const Mat3& m) {  // src/mesh.rs:419-428
    Mat3 r;
    r.xx = a.xx * m.xx + a.xy * m.yx + a.xz * m.zx; r.xy = a.xx * m.xy + a.xy * m.yy + a.xz * m.zy; r.xz = a.xx * m.xz + a.xy * m.yz + a.xz * m.zz;
    r.yx = a.yx * m.xx + a.yy * m.yx + a.yz * m.zx; r.yy = a.yx * m.xy + a.yy * m.yy + a.yz * m.zy; r.yz = a.yx * m.xz + a.yy * m.yz + a.yz * m.zz;
    r.zx = a.zx * m.xx + a.zy * m.yx + a.zz * m.zx; r.zy = a.zx * m.xy + a.zy * m.yy + a.zz * m.zy; r.zz = a.zx * m.xz + a.zy * m.yz + a.zz * m.zz;
    return r;
}
Mat3 rotation_deg(float rx, float ry, float rz) {  // construct_rotation_matrix, src/mesh.rs:51-55
    const float pi = (float)3.14159265358979323846;
    return matmul(matmul(rot_around(1, 0, 0, rx * pi / 180.0f), rot_around(0, 1, 0, ry * pi / 180.0f)),
                  rot_around(0, 0, 1, rz * pi / 180.0f));
}

int read_stl(const char* path, bool reposition, const float box[3], const float center[3], const Mat3& R, float size,
             HostMesh& mesh) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(ION_E_IO, "could not open or find file \"%s\"", path);
    std::vector<unsigned char> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    if (buf.size() < 84) return fail(ION_E_FORMAT, "\"%s\" is corrupted or unsupported (only binary .stl)", path);
    auto u32 = [&](size_t o) { return (uint32_t)buf[o] | ((uint32_t)buf[o + 1] << 8) | ((uint32_t)buf[o + 2] << 16) | ((uint32_t)buf[o + 3] << 24); };
    auto f32 = [&](size_t o) { const uint32_t u = u32(o); float v; memcpy(&v, &u, 4); return v; };
    const uint32_t nt = u32(80);
    if (nt == 0 || buf.size() != 84ull + 50ull * nt)
        return fail(ION_E_FORMAT, "\"%s\" is corrupted or unsupported (only binary .stl)", path);
    mesh = HostMesh();
    mesh.ntri = nt;
    mesh.p0.resize(3 * (size_t)nt); mesh.p1.resize(3 * (size_t)nt); mesh.p2.resize(3 * (size_t)nt);
    for (int a = 0; a < 3; a++) mesh.center[a] = center[a];
    size_t o = 84;
    for (uint32_t i = 0; i < nt; i++) {
        o += 12;  // normal
        float* dst[3] = {&mesh.p0[3 * (size_t)i], &mesh.p1[3 * (size_t)i], &mesh.p2[3 * (size_t)i]};
        for (int v = 0; v < 3; v++) {
            const float x = f32(o), y = f32(o + 4), z = f32(o + 8);
            o += 12;
            dst[v][0] = R.xx * x + R.xy * y + R.xz * z;
            dst[v][1] = R.yx * x + R.yy * y + R.yz * z;
            dst[v][2] = R.zx * x + R.zy * y + R.zz * z;
        }
        o += 2;  // attribute bits
    }
    mesh.update_bounds();
    float scale;
    if (size == 0.0f) {
        scale = std::fmin(box[0] / (mesh.pmax[0] - mesh.pmin[0]),
                          std::fmin(box[1] / (mesh.pmax[1] - mesh.pmin[1]), box[2] / (mesh.pmax[2] - mesh.pmin[2])));
    } else if (size > 0.0f) {
        const float mx = std::fmax(mesh.pmax[0] - mesh.pmin[0], std::fmax(mesh.pmax[1] - mesh.pmin[1], mesh.pmax[2] - mesh.pmin[2]));
        scale = size / mx;
    } else {
        scale = -size;
    }
    float off[3] = {0, 0, 0};
    if (reposition) for (int a = 0; a < 3; a++) off[a] = -0.5f * (mesh.pmin[a] + mesh.pmax[a]);
    for (std::vector<float>* p : {&mesh.p0, &mesh.p1, &mesh.p2})
        for (uint32_t i = 0; i < nt; i++)
            for (int a = 0; a < 3; a++) (*p)[3 * (size_t)i + a] = center[a] + scale * (off[a] + (*p)[3 * (size_t)i + a]);
    mesh.update_bounds();
    return ION_OK;
}

// -------- .ion byte stream (src/file.rs:336-433) ---------------------------
struct Reader {
    const std::vector<unsigned char>& b;
    size_t pos = 0;
    bool ok = true;
    bool need(size_t n) { if (pos + n > b.size()) ok = false; return ok; }
    uint8_t u8() { if (!need(1)) return 0; return b[pos++]; }
    uint32_t u32() { if (!need(4)) return 0; uint32_t v = 0; for (int i = 0; i < 4; i++) v |= (uint32_t)b[pos++] << (8 * i); return v; }
    float f32() { const uint32_t u = u32(); float f; memcpy(&f, &u, 4); return f; }
};
void push32(std::vector<unsigned char>& v, uint32_t x) { for (int i = 0; i < 4; i++) v.push_back((unsigned char)(x >> (8 * i))); }
void pushf(std::vector<unsigned char>& v, float f) { uint32_t u; memcpy(&u, &f, 4); push32(v, u); }

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int ion_abi_version(void) { return ION_ABI_VERSION; }
const char* ion_last_error(void) { return g_error.c_str(); }
uint64_t ion_kernel_launch_count(void) { return g_launches.load(); }

int ion_units_default(ion_units* u) {
    if (!u) return fail(ION_E_INVALID, "null units");
    u->m = 1.0f; u->kg = 1.0f; u->s = 1.0f; u->a = 1.0f; u->k = 1.0f; u->prop = ION_PROP_H;
    return ION_OK;
}

int ion_units_set(ion_units* u, float lbm_length, float lbm_velocity, float lbm_rho, float lbm_charge, float lbm_temp,
                  float si_length, float si_velocity, float si_rho, float si_charge, float si_temp) {
    if (!u) return fail(ION_E_INVALID, "null units");
    u->m = si_length / lbm_length;                  // src/lbm/units.rs:54-58
    u->kg = si_rho / lbm_rho * cbf(u->m);
    u->s = u->m / (si_velocity / lbm_velocity);
    u->a = si_charge / lbm_charge / u->s;
    u->k = si_temp / lbm_temp;
    return ION_OK;
}

int ion_units_si_to_lu(const ion_units* u, int what, float v, float* out) {
    if (!u || !out) return fail(ION_E_INVALID, "null argument");
    switch (what) {
        case 0: *out = v / (sqf(u->m) / u->s); break;  // nu_si_lu
        case 1: *out = v / (u->a / u->m); break;       // magnetization_si_lu
        case 2: *out = v / (u->a * u->s); break;       // charge_si_lu
        case 3: *out = v / u->m; break;                // len_si_lu
        default: return fail(ION_E_INVALID, "unknown conversion %d", what);
    }
    return ION_OK;
}

int ion_config_default(ion_config* c) {
    if (!c) return fail(ION_E_INVALID, "null config");
    memset(c, 0, sizeof *c);
    c->velocity_set = ION_D2Q9;
    c->relaxation_time = ION_SRT;
    c->float_type = ION_FP16S;
    ion_units_default(&c->units);
    c->n_x = c->n_y = c->n_z = 1;
    c->d_x = c->d_y = c->d_z = 1;
    c->nu = 1.0f / 6.0f;
    c->mhd_lod_depth = 4;
    c->update_fields = 1;  // graphics_active defaults to true (graphics.rs:160)
    c->field_mode = ION_FIELD_BITWISE;
    return ION_OK;
}

int ion_constants_from_config(const ion_config* c, ion_constants* k) {
    if (!c || !k) return fail(ION_E_INVALID, "null argument");
    derive_constants(*c, *k);
    return ION_OK;
}

int ion_lbm_create(const ion_config* cfg, ion_lbm** out) {
    if (!cfg || !out) return fail(ION_E_INVALID, "null argument");
    *out = nullptr;
    int rc = validate(*cfg);
    if (rc) return rc;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaFree(0) != cudaSuccess) {
        cudaGetLastError();
        return fail(ION_E_CUDA, "no usable CUDA device");
    }
    ion_lbm* h = new ion_lbm();
    h->cfg = *cfg;
    derive_constants(*cfg, h->k);
    h->q = velocity_q(cfg->velocity_set);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return fail(ION_E_CUDA, "cudaStreamCreate failed");
    }
    DevLbm& L = h->L;
    L.nx = cfg->n_x; L.ny = cfg->n_y; L.nz = cfg->n_z;
    L.n = cfg->n_x * cfg->n_y * cfg->n_z;
    L.dx = FastDiv(L.nx);
    L.dxy = FastDiv(L.nx * L.ny);
    const size_t N = L.n, db = ddf_bytes(cfg->float_type);
    const bool mhd = cfg->ext_magneto_hydro;
    auto A = [&](void** p, size_t bytes) { return rc ? rc : (rc = dmalloc(h, p, bytes)); };
    A(&L.fi, N * h->q * db);
    A((void**)&L.rho, N * 4);
    A((void**)&L.u, 3 * N * 4);
    A((void**)&L.flags, N);
    if (cfg->ext_force_field) A((void**)&L.F, 3 * N * 4);
    uint32_t depth = cfg->mhd_lod_depth, nd = 1u << depth;
    uint32_t n_lod_own = 1;
    for (uint32_t i = 0; i < depth; i++) n_lod_own += (1u << (i + 1)) * (1u << (i + 1)) * (1u << (i + 1));
    if (mhd) {
        const size_t npsi = (size_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
        h->e_dyn_count = npsi > 3 * N ? npsi : 3 * N;
        A((void**)&L.e_stat, 3 * N * 4);
        A((void**)&L.b_stat, 3 * N * 4);
        A((void**)&L.e_dyn, h->e_dyn_count * 4);
        A((void**)&L.b_dyn, 3 * N * 4);
        A(&L.fqi, 7 * N * db);
        A(&L.ei, N * h->q * db);
        A((void**)&L.q, N * 4);
        A((void**)&L.qu_lod, (size_t)n_lod_own * 16);
        if (depth > 0) A((void**)&L.lod_cell, 3 * N * 4);
        A((void**)&L.lod_pos, (size_t)n_lod_own * 16);
        if (cfg->ext_subgrid_ecr) {  // domain.rs:200-211
            A((void**)&L.e_var, 3 * N * 4);
            A(&L.eti, 7 * N * db);
            A((void**)&L.et, N * 4);
        }
    }
    A((void**)&h->d_err, 4);
    h->nparts = 1024;
    A((void**)&h->d_partials, h->nparts * sizeof(double));
    A((void**)&h->d_sums, 4 * sizeof(double));
    A((void**)&h->d_count, 2 * sizeof(uint32_t));
    if (rc) { destroy_handle(h); return rc; }
    k_fill<<<grid_for(N, 256), 256, 0, h->stream>>>(L.rho, N, 1.0f);  // rho starts at 1 (domain.rs:156)
    g_launches++;
    L.w = h->k.w; L.ke = h->k.ke; L.kmu = h->k.kmu; L.kmu0 = h->k.kmu0; L.kkge = h->k.kkge; L.wq = h->k.wq;
    L.kkbme = h->k.kkbme; L.keabs = h->k.keabs;
    L.rho_e0 = 0.0f;
    L.wait_limit = WAIT_LIMIT;
    L.fx = cfg->f_x; L.fy = cfg->f_y; L.fz = cfg->f_z;
    L.ext_eq = cfg->ext_equilibrium_boundaries; L.ext_vf = cfg->ext_volume_force; L.ext_ff = cfg->ext_force_field;
    L.ext_mhd = mhd; L.update_fields = cfg->update_fields; L.trt = cfg->relaxation_time == ION_TRT;
    L.depth = depth; L.nd = nd; L.n_lod_own = n_lod_own;
    L.n_bins = nd * nd * nd;
    L.first_src = n_lod_own > L.n_bins ? n_lod_own - L.n_bins : 0u;
    if (mhd) {
        L.bsx = L.nx / nd; L.bsy = L.ny / nd; L.bsz = L.nz / nd;
        L.ils = 1.0f / (float)(L.bsx * L.bsy * L.bsz);  // 1/lod_s(D), sim_kernels.cl:435-438, 672
        const uint32_t big = 1u << nd;                   // near block NX/(1<<(1<<D)), sim_kernels.cl:907-910
        L.near_x = std::max(L.nx / big, 1u); L.near_y = std::max(L.ny / big, 1u); L.near_z = std::max(L.nz / big, 1u);
        // LOD bin centres, lod_coordinates (sim_kernels.cl:440-447)
        std::vector<float4> pos(n_lod_own);
        const float dsx = (float)(L.nx / nd), dsy = (float)(L.ny / nd), dsz = (float)(L.nz / nd);
        for (uint32_t d = 0; d < n_lod_own; d++) {
            const uint32_t tt = d % (nd * nd);
            pos[d] = make_float4((float)(tt % nd) * dsx + (0.5f * dsx), (float)(tt / nd) * dsy + (0.5f * dsy),
                                 (float)(d / (nd * nd)) * dsz + (0.5f * dsz), 0.0f);
        }
        if (cudaMemcpyAsync(L.lod_pos, pos.data(), pos.size() * 16, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
            cudaStreamSynchronize(h->stream) != cudaSuccess) {
            destroy_handle(h);
            return fail(ION_E_CUDA, "upload of LOD centres failed");
        }
    }
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) { destroy_handle(h); return fail(ION_E_CUDA, "create: stream sync failed"); }
    for (auto& e : h->ev) cudaEventCreate(&e);
    *out = h;
    return ION_OK;
}

int ion_lbm_destroy(ion_lbm* h) {
    destroy_handle(h);
    return ION_OK;
}

int ion_lbm_get_config(const ion_lbm* h, ion_config* out) {
    if (!h || !out) return fail(ION_E_INVALID, "null argument");
    *out = h->cfg;
    return ION_OK;
}

int ion_lbm_initialize(ion_lbm* h) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    const int ft = h->cfg.float_type, mode = lbm_mode(h->cfg);
    const bool mhd = h->cfg.ext_magneto_hydro;
    h->t = 1;
    if (h->q == 19) q19_initialize(h->L, ft, mode, h->stream);
    else if (h->q == 15) q15_initialize(h->L, ft, mode, h->stream);
    else q9_initialize(h->L, ft, mode, h->stream);
    g_launches++;
    CKL();
    if (mhd) {
        int rc = launch_field(h);
        if (rc) return rc;
    }
    h->t = 0;
    h->initialized = true;
    return ION_OK;
}

int ion_lbm_set_electron_background(ion_lbm* h, float rho_e0) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    if (!h->cfg.ext_magneto_hydro) return fail(ION_E_STATE, "the electron background applies to ext_magneto_hydro");
    if (!(rho_e0 >= 0.0f) || !std::isfinite(rho_e0)) return fail(ION_E_INVALID, "rho_e0 must be finite and >= 0");
    h->L.rho_e0 = rho_e0;
    return ION_OK;
}

int ion_lbm_set_wait_limit(ion_lbm* h, uint32_t polls) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    h->L.wait_limit = polls;
    h->graph_dirty = true;  // the captured launches hold the old value
    return ION_OK;
}

int ion_lbm_do_time_step(ion_lbm* h) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    int rc = enqueue_step(h, h->t);
    if (rc) return rc;
    h->t += 1;
    return ION_OK;
}

int ion_lbm_run(ion_lbm* h, uint64_t steps) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    if (!h->initialized) {
        int rc = ion_lbm_initialize(h);
        if (rc) return rc;
    }
    if (h->ktiming || steps < 4) {
        for (uint64_t i = 0; i < steps; i++) {
            int rc = ion_lbm_do_time_step(h);
            if (rc) return rc;
        }
        return ION_OK;
    }
    if (h->t & 1u) {  // the graph holds an even step followed by an odd one
        int rc = ion_lbm_do_time_step(h);
        if (rc) return rc;
        steps--;
    }
    if (h->graph && h->graph_dirty) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    h->graph_dirty = false;
    if (!h->graph) {
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_step(h, 0);
        if (!rc) rc = enqueue_step(h, 1);
        cudaError_t e = cudaStreamEndCapture(h->stream, &g);
        if (rc) return rc;
        if (e != cudaSuccess) return fail(ION_E_CUDA, "graph capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&h->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { h->graph = nullptr; return fail(ION_E_CUDA, "graph instantiate: %s", cudaGetErrorString(e)); }
        h->graph_kernels = 2 * kernels_per_step(h);
        g_launches -= h->graph_kernels;  // capture does not launch
    }
    for (uint64_t i = 0; i + 1 < steps; i += 2) {
        CK(cudaGraphLaunch(h->graph, h->stream));
        g_launches += h->graph_kernels;
        h->t += 2;
    }
    if (steps & 1u) return ion_lbm_do_time_step(h);
    return ION_OK;
}

int ion_lbm_get_time_step(const ion_lbm* h, uint64_t* t) {
    if (!h || !t) return fail(ION_E_INVALID, "null argument");
    *t = h->t;
    return ION_OK;
}

int ion_lbm_finish_queues(ion_lbm* h, int timeout_ms) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const cudaError_t e = cudaStreamQuery(h->stream);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) return fail(ION_E_CUDA, "stream: %s", cudaGetErrorString(e));
        if (timeout_ms >= 0 && std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(timeout_ms))
            return fail(ION_E_TIMEOUT, "stream still busy after %d ms", timeout_ms);
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    return h->cfg.ext_magneto_hydro ? check_device_error(h) : ION_OK;
}

int ion_lbm_update_fields(ion_lbm* h) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    const int ft = h->cfg.float_type;
    if (h->q == 19) q19_update_fields(h->L, ft, h->t, h->stream);
    else if (h->q == 15) q15_update_fields(h->L, ft, h->t, h->stream);
    else q9_update_fields(h->L, ft, h->t, h->stream);
    g_launches++;
    CKL();
    return ION_OK;
}

static void* field_ptr(ion_lbm* h, int f, size_t* eb, size_t* count) {
    const size_t N = h->L.n, db = ddf_bytes(h->cfg.float_type);
    const bool mhd = h->cfg.ext_magneto_hydro;
    void* p = nullptr;
    size_t e = 4, c = 0;
    switch (f) {
        case ION_FIELD_FI: p = h->L.fi; e = db; c = N * h->q; break;
        case ION_FIELD_RHO: p = h->L.rho; c = N; break;
        case ION_FIELD_U: p = h->L.u; c = 3 * N; break;
        case ION_FIELD_FLAGS: p = h->L.flags; e = 1; c = N; break;
        case ION_FIELD_F: p = h->L.F; c = h->L.F ? 3 * N : 0; break;
        case ION_FIELD_E_STAT: p = h->L.e_stat; c = mhd ? 3 * N : 0; break;
        case ION_FIELD_B_STAT: p = h->L.b_stat; c = mhd ? 3 * N : 0; break;
        case ION_FIELD_E_DYN: p = h->L.e_dyn; c = mhd ? h->e_dyn_count : 0; break;
        case ION_FIELD_B_DYN: p = h->L.b_dyn; c = mhd ? 3 * N : 0; break;
        case ION_FIELD_FQI: p = h->L.fqi; e = db; c = mhd ? 7 * N : 0; break;
        case ION_FIELD_EI: p = h->L.ei; e = db; c = mhd ? N * h->q : 0; break;
        case ION_FIELD_Q: p = h->L.q; c = mhd ? N : 0; break;
        case ION_FIELD_QU_LOD: p = h->L.qu_lod; c = mhd ? 4 * (size_t)h->L.n_lod_own : 0; break;
        case ION_FIELD_E_VAR: p = h->L.e_var; c = h->L.e_var ? 3 * N : 0; break;
        case ION_FIELD_ETI: p = h->L.eti; e = db; c = h->L.eti ? 7 * N : 0; break;
        case ION_FIELD_ET: p = h->L.et; c = h->L.et ? N : 0; break;
        default: break;
    }
    if (eb) *eb = e;
    if (count) *count = c;
    return c ? p : nullptr;
}

int ion_lbm_field_info(const ion_lbm* h, int field, size_t* elem_bytes, size_t* count) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    if (field < 0 || field >= ION_FIELD_COUNT) return fail(ION_E_INVALID, "unknown field %d", field);
    field_ptr(const_cast<ion_lbm*>(h), field, elem_bytes, count);
    return ION_OK;
}

int ion_lbm_write_field(ion_lbm* h, int field, const void* host, size_t bytes) {
    if (!h || !host) return fail(ION_E_INVALID, "null argument");
    size_t eb, c;
    void* p = field_ptr(h, field, &eb, &c);
    if (!p) return fail(ION_E_INVALID, "field %d is not present in this configuration", field);
    if (bytes > eb * c) return fail(ION_E_INVALID, "field %d holds %zu bytes, got %zu", field, eb * c, bytes);
    CK(cudaMemcpyAsync(p, host, bytes, cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return ION_OK;
}

int ion_lbm_read_field(ion_lbm* h, int field, void* host, size_t bytes) {
    if (!h || !host) return fail(ION_E_INVALID, "null argument");
    size_t eb, c;
    void* p = field_ptr(h, field, &eb, &c);
    if (!p) return fail(ION_E_INVALID, "field %d is not present in this configuration", field);
    if (bytes > eb * c) return fail(ION_E_INVALID, "field %d holds %zu bytes, asked for %zu", field, eb * c, bytes);
    CK(cudaMemcpyAsync(host, p, bytes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return h->cfg.ext_magneto_hydro ? check_device_error(h) : ION_OK;
}

int ion_lbm_field_device_ptr(ion_lbm* h, int field, void** dptr, size_t* bytes) {
    if (!h || !dptr) return fail(ION_E_INVALID, "null argument");
    size_t eb, c;
    *dptr = field_ptr(h, field, &eb, &c);
    if (bytes) *bytes = eb * c;
    return *dptr ? ION_OK : fail(ION_E_INVALID, "field %d is not present", field);
}

int ion_lbm_stream(ion_lbm* h, void** s) {
    if (!h || !s) return fail(ION_E_INVALID, "null argument");
    *s = (void*)h->stream;
    return ION_OK;
}

// ---- meshes ----------------------------------------------------------------
int ion_lbm_add_mesh(ion_lbm* h, const float* p0, const float* p1, const float* p2, uint32_t ntri, uint32_t* index) {
    if (!h || !p0 || !p1 || !p2 || ntri == 0) return fail(ION_E_INVALID, "empty or null mesh");
    HostMesh m;
    m.ntri = ntri;
    m.p0.assign(p0, p0 + 3 * (size_t)ntri);
    m.p1.assign(p1, p1 + 3 * (size_t)ntri);
    m.p2.assign(p2, p2 + 3 * (size_t)ntri);
    m.update_bounds();
    for (int a = 0; a < 3; a++) m.center[a] = 0.5f * (m.pmin[a] + m.pmax[a]);
    h->meshes.push_back(std::move(m));
    if (index) *index = (uint32_t)h->meshes.size() - 1;
    return ION_OK;
}

int ion_lbm_import_mesh(ion_lbm* h, const char* path, float scale, float ox, float oy, float oz, float rx, float ry,
                        float rz, uint32_t* index) {
    if (!h || !path) return fail(ION_E_INVALID, "null argument");
    const float box[3] = {1.0f, 1.0f, 1.0f}, c[3] = {ox, oy, oz};
    const float scale_lu = scale / h->cfg.units.m;  // len_si_lu
    HostMesh m;
    int rc = read_stl(path, false, box, c, rotation_deg(rx, ry, rz), -std::fabs(scale_lu), m);
    if (rc) return rc;
    h->meshes.push_back(std::move(m));
    if (index) *index = (uint32_t)h->meshes.size() - 1;
    return ION_OK;
}

int ion_lbm_import_mesh_reposition(ion_lbm* h, const char* path, float cx, float cy, float cz, float rx, float ry,
                                   float rz, float size, uint32_t* index) {
    if (!h || !path) return fail(ION_E_INVALID, "null argument");
    const float box[3] = {(float)h->cfg.n_x, (float)h->cfg.n_y, (float)h->cfg.n_z}, c[3] = {cx, cy, cz};
    HostMesh m;
    int rc = read_stl(path, true, box, c, rotation_deg(rx, ry, rz), size, m);
    if (rc) return rc;
    h->meshes.push_back(std::move(m));
    if (index) *index = (uint32_t)h->meshes.size() - 1;
    return ION_OK;
}

int ion_lbm_mesh_translate(ion_lbm* h, uint32_t index, float dx, float dy, float dz) {
    if (!h || index >= h->meshes.size()) return fail(ION_E_INVALID, "no mesh %u", index);
    HostMesh& m = h->meshes[index];
    const float d[3] = {dx, dy, dz};
    for (std::vector<float>* p : {&m.p0, &m.p1, &m.p2})
        for (uint32_t i = 0; i < m.ntri; i++)
            for (int a = 0; a < 3; a++) (*p)[3 * (size_t)i + a] += d[a];
    for (int a = 0; a < 3; a++) { m.center[a] += d[a]; m.pmin[a] += d[a]; m.pmax[a] += d[a]; }
    return ION_OK;
}

int ion_lbm_mesh_triangles(const ion_lbm* h, uint32_t index, float* p0, float* p1, float* p2, uint32_t capacity,
                           uint32_t* ntri) {
    if (!h || index >= h->meshes.size()) return fail(ION_E_INVALID, "no mesh %u", index);
    const HostMesh& m = h->meshes[index];
    if (ntri) *ntri = m.ntri;
    if (!p0 && !p1 && !p2) return ION_OK;  // size query
    if (!p0 || !p1 || !p2 || capacity < m.ntri) return fail(ION_E_INVALID, "mesh %u has %u triangles", index, m.ntri);
    memcpy(p0, m.p0.data(), sizeof(float) * 3 * (size_t)m.ntri);
    memcpy(p1, m.p1.data(), sizeof(float) * 3 * (size_t)m.ntri);
    memcpy(p2, m.p2.data(), sizeof(float) * 3 * (size_t)m.ntri);
    return ION_OK;
}

int ion_lbm_mesh_bounds(const ion_lbm* h, uint32_t index, float* out9) {
    if (!h || !out9 || index >= h->meshes.size()) return fail(ION_E_INVALID, "no mesh %u", index);
    const HostMesh& m = h->meshes[index];
    for (int a = 0; a < 3; a++) { out9[a] = m.pmin[a]; out9[3 + a] = m.pmax[a]; out9[6 + a] = m.center[a]; }
    return ION_OK;
}

// Lbm::voxelise_mesh -> LbmDomain::voxelize_mesh_on_device (src/mesh.rs:256-343)
int ion_lbm_voxelise_mesh(ion_lbm* h, uint32_t index, int model_type, float v0, float v1, float v2) {
    if (!h || index >= h->meshes.size()) return fail(ION_E_INVALID, "no mesh %u", index);
    const HostMesh& m = h->meshes[index];
    const size_t need = 3 * (size_t)m.ntri;
    if (need > h->tri_cap) {
        void* p;
        int rc = 0;
        if ((rc = dmalloc(h, &p, need * 4))) return rc;
        h->d_p0 = (float*)p;
        if ((rc = dmalloc(h, &p, need * 4))) return rc;
        h->d_p1 = (float*)p;
        if ((rc = dmalloc(h, &p, need * 4))) return rc;
        h->d_p2 = (float*)p;
        h->tri_cap = need;
    }
    CK(cudaMemcpyAsync(h->d_p0, m.p0.data(), need * 4, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_p1, m.p1.data(), need * 4, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_p2, m.p2.data(), need * 4, cudaMemcpyHostToDevice, h->stream));
    VoxArgs A{};
    A.p0 = h->d_p0; A.p1 = h->d_p1; A.p2 = h->d_p2; A.ntri = m.ntri;
    A.x0 = m.pmin[0] - 2.0f; A.y0 = m.pmin[1] - 2.0f; A.z0 = m.pmin[2] - 2.0f;
    A.x1 = m.pmax[0] + 2.0f; A.y1 = m.pmax[1] + 2.0f; A.z1 = m.pmax[2] + 2.0f;
    const float c0 = (A.y1 - A.y0) * (A.z1 - A.z0), c1 = (A.z1 - A.z0) * (A.x1 - A.x0), c2 = (A.x1 - A.x0) * (A.y1 - A.y0);
    A.direction = (c0 < c1 && c0 < c2) ? 0 : (c1 < c2 ? 1 : 2);
    const uint32_t area[3] = {h->L.ny * h->L.nz, h->L.nx * h->L.nz, h->L.nx * h->L.ny};
    A.columns = area[A.direction];
    const ion_units& u = h->cfg.units;
    switch (model_type) {
        case ION_MODEL_SOLID: A.flag = 0x01; break;
        case ION_MODEL_MAGNET: A.flag = 0x11; A.mx = v0 / (u.a / u.m); A.my = v1 / (u.a / u.m); A.mz = v2 / (u.a / u.m); break;
        case ION_MODEL_CHARGED: A.flag = 0x09; A.mx = v0 / (u.a * u.s); break;
        case ION_MODEL_CHARGED_ECR: A.flag = 0x05; A.mx = v0 / (u.a * u.s); break;
        default: return fail(ION_E_INVALID, "unknown model type %d", model_type);
    }
    launch_voxelize(h->L, A, h->stream);
    g_launches++;
    CKL();
    CK(cudaStreamSynchronize(h->stream));  // the host triangle arrays may change after return
    return ION_OK;
}

static int ensure_compaction(ion_lbm* h) {
    if (h->d_list) return ION_OK;
    void* p;
    int rc = dmalloc(h, &p, sizeof(uint32_t) * (((size_t)h->L.n + 1023) / 1024 + 1));
    if (rc) return rc;
    h->d_tiles = (uint32_t*)p;
    rc = dmalloc(h, &p, sizeof(uint32_t) * (size_t)h->L.n);
    if (rc) return rc;
    h->d_list = (uint32_t*)p;
    return ION_OK;
}

int ion_lbm_precompute_b(ion_lbm* h) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    if (!h->cfg.ext_magneto_hydro) return fail(ION_E_STATE, "precompute_b needs ext_magneto_hydro");
    int rc = ensure_compaction(h);
    if (rc) return rc;
    launch_compact(h->L, F_M, h->d_tiles, h->d_list, h->d_count, h->stream);
    g_launches += 3;
    launch_psi_static_b(h->L, h->d_list, h->d_count, h->stream);
    g_launches += 2;
    CKL();
    CK(cudaStreamSynchronize(h->stream));
    return ION_OK;
}

int ion_lbm_precompute_e(ion_lbm* h) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    if (!h->cfg.ext_magneto_hydro) return fail(ION_E_STATE, "precompute_e needs ext_magneto_hydro");
    int rc = ensure_compaction(h);
    if (rc) return rc;
    launch_compact(h->L, F_F | F_C, h->d_tiles, h->d_list, h->d_count, h->stream);
    g_launches += 3;
    launch_static_e(h->L, h->d_list, h->d_count, h->L.e_stat, h->stream);
    g_launches++;
    CKL();
    CK(cudaStreamSynchronize(h->stream));
    return ION_OK;
}

int ion_lbm_precompute_e_ecr(ion_lbm* h) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    if (!h->cfg.ext_magneto_hydro || !h->cfg.ext_subgrid_ecr)
        return fail(ION_E_STATE, "precompute_e_ecr needs ext_magneto_hydro and ext_subgrid_ecr");
    int rc = ensure_compaction(h);
    if (rc) return rc;
    launch_compact(h->L, F_F | F_C, h->d_tiles, h->d_list, h->d_count, h->stream);
    g_launches += 3;
    launch_static_e(h->L, h->d_list, h->d_count, h->L.e_var, h->stream);  // domain.rs:569-578
    g_launches++;
    CKL();
    CK(cudaStreamSynchronize(h->stream));
    return ION_OK;
}

int ion_lbm_mass_charge(ion_lbm* h, double* mass, double* charge) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    const size_t N = h->L.n;
    const int ft = h->cfg.float_type;
    launch_sum_f64(h->L.fi, ft, N * h->q, h->d_partials, h->nparts, h->d_sums + 0, h->stream);
    g_launches += 2;
    if (h->cfg.ext_magneto_hydro) {
        launch_sum_f64(h->L.fqi, ft, N * 7, h->d_partials, h->nparts, h->d_sums + 1, h->stream);
        launch_sum_f64(h->L.ei, ft, N * h->q, h->d_partials, h->nparts, h->d_sums + 2, h->stream);
        g_launches += 4;
    }
    CKL();
    double s[3] = {0, 0, 0};
    CK(cudaMemcpyAsync(s, h->d_sums, sizeof s, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    // DDFs are stored shifted by -w_i (sum_i w_i = 1 per cell): add N back
    if (mass) *mass = s[0] + (double)N;
    if (charge) *charge = h->cfg.ext_magneto_hydro ? (s[1] + (double)N) - (s[2] + (double)N) : 0.0;
    return ION_OK;
}

// ---- .ion files (src/file.rs:42-306, FILE_LAYOUT.txt) -----------------------
int ion_lbm_save(ion_lbm* h, const char* path) {
    if (!h || !path) return fail(ION_E_INVALID, "null argument");
    const ion_config& c = h->cfg;
    const size_t N = h->L.n;
    std::vector<unsigned char> b;
    const char* hdr = "IonSolver setup\n";
    b.insert(b.end(), hdr, hdr + 16);
    b.push_back((unsigned char)c.velocity_set);
    b.push_back((unsigned char)c.relaxation_time);
    b.push_back((unsigned char)c.float_type);
    pushf(b, c.units.m); pushf(b, c.units.kg); pushf(b, c.units.s); pushf(b, c.units.a);
    push32(b, c.n_x); push32(b, c.n_y); push32(b, c.n_z);
    b.push_back(0);  // fixed domains
    push32(b, c.d_x); push32(b, c.d_y); push32(b, c.d_z);
    pushf(b, c.nu); pushf(b, c.f_x); pushf(b, c.f_y); pushf(b, c.f_z);
    b.push_back((unsigned char)((c.ext_equilibrium_boundaries ? 1 : 0) | (c.ext_volume_force ? 2 : 0) |
                                (c.ext_force_field ? 4 : 0) | (c.ext_magneto_hydro ? 8 : 0)));
    b.push_back(c.mhd_lod_depth);
    const size_t head = b.size();
    b.resize(head + N + 16 * N + (c.ext_magneto_hydro ? 4 * N : 0));
    int rc = ion_lbm_read_field(h, ION_FIELD_FLAGS, b.data() + head, N);
    if (!rc) rc = ion_lbm_read_field(h, ION_FIELD_RHO, b.data() + head + N, 4 * N);
    if (!rc) rc = ion_lbm_read_field(h, ION_FIELD_U, b.data() + head + 5 * N, 12 * N);
    if (!rc && c.ext_magneto_hydro) rc = ion_lbm_read_field(h, ION_FIELD_Q, b.data() + head + 17 * N, 4 * N);
    if (rc) return rc;
    // floats are little-endian on both supported hosts (x86-64, aarch64)
    std::ofstream f(path, std::ios::binary);
    if (!f) return fail(ION_E_IO, "writing went wrong: cannot open \"%s\"", path);
    f.write((const char*)b.data(), (std::streamsize)b.size());
    if (!f) return fail(ION_E_IO, "writing went wrong: \"%s\"", path);
    return ION_OK;
}

int ion_lbm_load(const char* path, ion_config* cfg, ion_lbm** out) {
    if (!path || !cfg || !out) return fail(ION_E_INVALID, "null argument");
    *out = nullptr;
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(ION_E_IO, "Could not find file.");
    std::vector<unsigned char> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    Reader r{buf};
    char hdr[17] = {0};
    for (int i = 0; i < 16; i++) hdr[i] = (char)r.u8();
    if (!r.ok || strcmp(hdr, "IonSolver setup\n") != 0) return fail(ION_E_FORMAT, "Invalid Format!");
    ion_config c = *cfg;
    c.velocity_set = r.u8();
    c.relaxation_time = r.u8();
    c.float_type = r.u8();  // FloatType discriminants of types.rs:75-83 (the encoder's mapping)
    c.units.m = r.f32(); c.units.kg = r.f32(); c.units.s = r.f32(); c.units.a = r.f32();
    c.n_x = r.u32(); c.n_y = r.u32(); c.n_z = r.u32();
    r.u8();  // fixed domains: skipped, as in the reference
    c.d_x = r.u32(); c.d_y = r.u32(); c.d_z = r.u32();
    c.nu = r.f32(); c.f_x = r.f32(); c.f_y = r.f32(); c.f_z = r.f32();
    const uint8_t ext = r.u8();
    c.ext_equilibrium_boundaries = (ext & 1) != 0;
    c.ext_volume_force = (ext & 2) != 0;
    c.ext_force_field = (ext & 4) != 0;
    c.ext_magneto_hydro = (ext & 8) != 0;
    c.mhd_lod_depth = r.u8();
    if (!r.ok) return fail(ION_E_FORMAT, "file truncated in the config block");
    int vrc = validate(c);  // before the body size is formed from the dimensions
    if (vrc) return vrc;
    const uint64_t N = (uint64_t)c.n_x * c.n_y * c.n_z;
    const uint64_t body = N * 17 + (c.ext_magneto_hydro ? 4 * N : 0);
    if (buf.size() - r.pos < body) return fail(ION_E_FORMAT, "Not all data could be read, file may be corrupted.");
    const size_t o = r.pos;
    r.pos += body;
    const bool ext_block = buf.size() - r.pos >= 4 && memcmp(buf.data() + r.pos, "IONX", 4) == 0;
    if (ext_block) {
        r.pos = buf.size();  // a checkpoint's extension block: read as a plain .ion file here
    } else if (c.ext_magneto_hydro && r.pos != buf.size()) {
        // fixed charges and magnets (FILE_LAYOUT.txt:46-58): read and discarded,
        // as the reference does; the reference's writer omits both sections.
        const uint32_t nc = r.u32();
        if (r.ok) r.pos += 12ull * nc;
        const uint32_t nm = r.ok && r.pos <= buf.size() ? r.u32() : 0;
        if (r.ok) r.pos += 20ull * nm;
        if (!r.ok || r.pos > buf.size()) return fail(ION_E_FORMAT, "Not all data could be read, file may be corrupted.");
    }
    if (r.pos != buf.size()) return fail(ION_E_FORMAT, "Not all data could be read, file may be corrupted.");
    ion_lbm* h = nullptr;
    int rc = ion_lbm_create(&c, &h);
    if (rc) return rc;
    rc = ion_lbm_write_field(h, ION_FIELD_FLAGS, buf.data() + o, N);
    if (!rc) rc = ion_lbm_write_field(h, ION_FIELD_RHO, buf.data() + o + N, 4 * N);
    if (!rc) rc = ion_lbm_write_field(h, ION_FIELD_U, buf.data() + o + 5 * N, 12 * N);
    if (!rc && c.ext_magneto_hydro) rc = ion_lbm_write_field(h, ION_FIELD_Q, buf.data() + o + 17 * N, 4 * N);
    if (rc) { destroy_handle(h); return rc; }
    *cfg = c;
    *out = h;
    return ION_OK;
}

// ---- full checkpoint ------------------------------------------------------------
// Extension block after the .ion image: "IONX", u32 version (1), u64 time step,
// u8 update_fields, u8 field_mode, u8 propellant, u8 0, f32 units.k, u32 section
// count, then per section u32 field id, u64 bytes, the raw device contents.
namespace {
const int kCheckpointFields[] = {ION_FIELD_FI,  ION_FIELD_F,     ION_FIELD_E_STAT, ION_FIELD_B_STAT,
                                 ION_FIELD_E_DYN, ION_FIELD_B_DYN, ION_FIELD_FQI,  ION_FIELD_EI,
                                 ION_FIELD_QU_LOD, ION_FIELD_E_VAR, ION_FIELD_ETI, ION_FIELD_ET};
}

int ion_lbm_checkpoint(ion_lbm* h, const char* path) {
    if (!h || !path) return fail(ION_E_INVALID, "null argument");
    if (!h->initialized) return fail(ION_E_STATE, "checkpoint of a handle that was not initialized");
    int rc = ion_lbm_save(h, path);
    if (rc) return rc;
    std::vector<unsigned char> b;
    const char* magic = "IONX";
    b.insert(b.end(), magic, magic + 4);
    push32(b, 1u);
    push32(b, (uint32_t)(h->t & 0xFFFFFFFFu));
    push32(b, (uint32_t)(h->t >> 32));
    b.push_back(h->cfg.update_fields);
    b.push_back(h->cfg.field_mode);
    b.push_back((unsigned char)h->cfg.units.prop);
    b.push_back(0);
    pushf(b, h->cfg.units.k);
    std::vector<std::pair<int, size_t>> secs;
    for (int id : kCheckpointFields) {
        size_t eb = 0, cnt = 0;
        if (ion_lbm_field_info(h, id, &eb, &cnt) == ION_OK && eb * cnt > 0) secs.push_back({id, eb * cnt});
    }
    push32(b, (uint32_t)secs.size());
    for (auto& sc : secs) {
        push32(b, (uint32_t)sc.first);
        push32(b, (uint32_t)(sc.second & 0xFFFFFFFFu));
        push32(b, (uint32_t)((uint64_t)sc.second >> 32));
        const size_t at = b.size();
        b.resize(at + sc.second);
        rc = ion_lbm_read_field(h, sc.first, b.data() + at, sc.second);
        if (rc) return rc;
    }
    std::ofstream f(path, std::ios::binary | std::ios::app);
    if (!f) return fail(ION_E_IO, "writing went wrong: cannot open \"%s\"", path);
    f.write((const char*)b.data(), (std::streamsize)b.size());
    if (!f) return fail(ION_E_IO, "writing went wrong: \"%s\"", path);
    return ION_OK;
}

int ion_lbm_restore(const char* path, ion_config* cfg, ion_lbm** out) {
    if (!path || !cfg || !out) return fail(ION_E_INVALID, "null argument");
    *out = nullptr;
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(ION_E_IO, "Could not find file.");
    std::vector<unsigned char> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    // locate the extension block: it follows the .ion body, whose size the header gives
    if (buf.size() < 16 + 62) return fail(ION_E_FORMAT, "Invalid Format!");
    Reader hr{buf};
    hr.pos = 16 + 3 + 16;
    const uint32_t nx = hr.u32(), ny = hr.u32(), nz = hr.u32();
    hr.pos = 16 + 62 - 2;
    const bool mhd = (hr.u8() & 8) != 0;
    const uint64_t nxy = (uint64_t)nx * ny;
    if (nxy >= (1ull << 32) || nxy * nz >= (1ull << 32)) return fail(ION_E_FORMAT, "grid of 2^32 or more cells");
    const uint64_t N = nxy * nz;
    const uint64_t ext_at = 16 + 62 + N * 17 + (mhd ? 4 * N : 0);
    if (!hr.ok || ext_at + 4 > buf.size() || memcmp(buf.data() + ext_at, "IONX", 4) != 0)
        return fail(ION_E_FORMAT, "\"%s\" is not a checkpoint (no extension block)", path);
    Reader r{buf};
    r.pos = ext_at + 4;
    const uint32_t version = r.u32();
    const uint64_t t = (uint64_t)r.u32() | ((uint64_t)r.u32() << 32);
    const uint8_t update_fields = r.u8(), field_mode = r.u8(), prop = r.u8();
    r.u8();
    const float unit_k = r.f32();
    const uint32_t nsec = r.u32();
    if (!r.ok || version != 1u) return fail(ION_E_FORMAT, "unsupported checkpoint version");
    ion_config c = *cfg;
    c.update_fields = update_fields;
    c.field_mode = field_mode;
    c.units.prop = prop;
    c.units.k = unit_k;
    ion_lbm* h = nullptr;
    int rc = ion_lbm_load(path, &c, &h);
    if (rc) return rc;
    for (uint32_t k = 0; k < nsec && !rc; k++) {
        const uint32_t id = r.u32();
        const uint64_t bytes = (uint64_t)r.u32() | ((uint64_t)r.u32() << 32);
        if (!r.ok || buf.size() - r.pos < bytes) { rc = fail(ION_E_FORMAT, "checkpoint truncated"); break; }
        size_t eb = 0, cnt = 0;
        if (ion_lbm_field_info(h, (int)id, &eb, &cnt) != ION_OK || eb * cnt != bytes) {
            rc = fail(ION_E_FORMAT, "checkpoint section %u does not match the configuration", id);
            break;
        }
        rc = ion_lbm_write_field(h, (int)id, buf.data() + r.pos, (size_t)bytes);
        r.pos += bytes;
    }
    if (!rc && r.pos != buf.size()) rc = fail(ION_E_FORMAT, "Not all data could be read, file may be corrupted.");
    if (!rc && cudaStreamSynchronize(h->stream) != cudaSuccess) rc = fail(ION_E_CUDA, "restore");
    if (rc) { destroy_handle(h); return rc; }
    h->t = t;
    h->initialized = true;
    h->graph_dirty = true;
    *cfg = c;
    *out = h;
    return ION_OK;
}

// ---- timing ------------------------------------------------------------------
int ion_lbm_record_event(ion_lbm* h, int slot) {
    if (!h || slot < 0 || slot >= 8) return fail(ION_E_INVALID, "bad event slot");
    CK(cudaEventRecord(h->ev[slot], h->stream));
    return ION_OK;
}

int ion_lbm_event_elapsed(ion_lbm* h, int a, int b, float* ms) {
    if (!h || !ms || a < 0 || a >= 8 || b < 0 || b >= 8) return fail(ION_E_INVALID, "bad event slot");
    CK(cudaEventSynchronize(h->ev[b]));
    CK(cudaEventElapsedTime(ms, h->ev[a], h->ev[b]));
    return ION_OK;
}

int ion_lbm_set_kernel_timing(ion_lbm* h, int enable) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    h->ktiming = enable != 0;
    return ION_OK;
}

int ion_lbm_kernel_time(ion_lbm* h, int kernel, double* total_ms, uint64_t* launches) {
    if (!h || kernel < 0 || kernel > 2) return fail(ION_E_INVALID, "bad kernel id");
    if (!h->kev.empty()) {
        CK(cudaStreamSynchronize(h->stream));
        for (auto& e : h->kev) {
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, e.a, e.b));
            h->ktime[e.kernel] += ms;
            h->kcount[e.kernel] += 1;
            h->ev_pool.push_back(e.a);
            h->ev_pool.push_back(e.b);
        }
        h->kev.clear();
    }
    if (total_ms) *total_ms = h->ktime[kernel];
    if (launches) *launches = h->kcount[kernel];
    return ION_OK;
}

int ion_lbm_reset_kernel_time(ion_lbm* h) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    double d;
    uint64_t c;
    int rc = ion_lbm_kernel_time(h, 0, &d, &c);
    if (rc) return rc;
    for (int i = 0; i < 3; i++) { h->ktime[i] = 0; h->kcount[i] = 0; }
    return ION_OK;
}

// ---- batches of independent domains (batch_kernels.cu) -----------------------
}  // extern "C"

namespace {
constexpr uint32_t BARRIER_LIMIT = 1u << 26;  // polls (64 ns apart) before a grid barrier gives up
static_assert(BARRIER_LIMIT == ION_BARRIER_LIMIT_DEFAULT && WAIT_LIMIT == ION_WAIT_LIMIT_DEFAULT,
              "the header's documented defaults");
}

struct ion_batch {
    std::vector<ion_lbm*> doms;
    int ft = ION_FP32;
    bool mhd = false, fast = false;
    cudaStream_t stream = nullptr;
    DevLbm* d_doms = nullptr;
    uint32_t* d_tile_off[3] = {nullptr, nullptr, nullptr};  // block 128, 256, 512
    uint32_t total_tiles[3] = {0, 0, 0};
    uint32_t* d_brick_off[3] = {nullptr, nullptr, nullptr};  // E/B tiles (bricks x 256 / block)
    uint32_t total_bricks[3] = {0, 0, 0};
    uint32_t* d_bin_off = nullptr;
    uint32_t total_bins = 0;
    uint32_t* d_row_off = nullptr;  // row-staged stencil: prefix sums of ny nz (null: tiles of cells)
    uint32_t total_rows = 0;
    uint32_t* d_sync = nullptr;  // [0] barrier count, [1] barrier generation, [2] error
    uint32_t barrier_limit = BARRIER_LIMIT;
    uint64_t t = 0;
    int sms = 0;
    bool tuned = false;
    uint32_t block = 256, grid = 0;
    std::vector<std::array<float, 3>> tuning;  // block, grid, ms per step
    cudaGraphExec_t graph = nullptr;
    bool graph_failed = false;
    cudaEvent_t ev[4] = {};
    std::vector<void*> allocs;
};

namespace {

const uint32_t kBatchBlocks[2] = {128, 256};

int block_slot(uint32_t block) { return block == 128 ? 0 : block == 256 ? 1 : 2; }

BatchDev batch_view(ion_batch* b, uint32_t block) {
    BatchDev B{};
    B.doms = b->d_doms;
    B.ndom = (uint32_t)b->doms.size();
    B.tile_off = b->d_tile_off[block_slot(BATCH_SC_THREADS)];  // the stencil kernel's block size
    B.total_tiles = b->total_tiles[block_slot(BATCH_SC_THREADS)];
    B.brick_off = b->d_brick_off[block_slot(block)];
    B.total_bricks = b->total_bricks[block_slot(block)];
    B.bin_off = b->d_bin_off;
    B.total_bins = b->total_bins;
    B.bar_count = b->d_sync;
    B.bar_gen = b->d_sync + 1;
    B.err = b->d_sync + 2;
    B.barrier_limit = b->barrier_limit;
    B.row_off = b->d_row_off;
    B.total_rows = b->total_rows;
    return B;
}

int batch_launch(ion_batch* b, uint32_t block, uint32_t grid) {
    const cudaError_t e = launch_batch_step(batch_view(b, block), b->ft, b->mhd, b->fast, grid, block, b->t, b->stream);
    if (e != cudaSuccess) return fail(ION_E_CUDA, "batch step launch: %s", cudaGetErrorString(e));
    g_launches += b->mhd ? 2 : 1;
    b->t += 1;
    return ION_OK;
}

void destroy_batch(ion_batch* b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (void* p : b->allocs) cudaFree(p);
    for (auto& e : b->ev) if (e) cudaEventDestroy(e);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

}  // namespace

extern "C" {

int ion_batch_create(ion_lbm* const* domains, uint32_t count, ion_batch** out) {
    if (!domains || !out || count == 0) return fail(ION_E_INVALID, "empty batch");
    *out = nullptr;
    ion_lbm* d0 = domains[0];
    for (uint32_t i = 0; i < count; i++) {
        ion_lbm* h = domains[i];
        if (!h) return fail(ION_E_INVALID, "null domain %u", i);
        if (h->q != 19) return fail(ION_E_CONFIG, "batches run D3Q19 domains");
        if (h->cfg.ext_subgrid_ecr) return fail(ION_E_CONFIG, "batches do not run the SUBGRID_ECR extension");
        if (h->cfg.float_type != d0->cfg.float_type || h->cfg.ext_magneto_hydro != d0->cfg.ext_magneto_hydro ||
            (h->cfg.ext_magneto_hydro && h->cfg.field_mode != d0->cfg.field_mode))
            return fail(ION_E_CONFIG, "domain %u differs from domain 0 in float type, MHD or field mode", i);
        for (uint32_t k = 0; k < i; k++)
            if (domains[k] == h) return fail(ION_E_INVALID, "domain %u appears twice", i);
    }
    for (uint32_t i = 0; i < count; i++) {
        ion_lbm* h = domains[i];
        if (!h->initialized) {
            int rc = ion_lbm_initialize(h);
            if (rc) return rc;
        }
        CK(cudaStreamSynchronize(h->stream));
        if ((h->t & 1u) != (d0->t & 1u)) return fail(ION_E_STATE, "domains must be at time steps of equal parity");
    }
    ion_batch* b = new ion_batch();
    b->doms.assign(domains, domains + count);
    b->ft = d0->cfg.float_type;
    b->mhd = d0->cfg.ext_magneto_hydro;
    b->fast = b->mhd && d0->cfg.field_mode == ION_FIELD_FAST;
    b->t = d0->t;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        return fail(ION_E_CUDA, "cudaStreamCreate failed");
    }
    auto dalloc = [&](void** p, size_t bytes) -> int {
        if (cudaMalloc(p, bytes) != cudaSuccess) { cudaGetLastError(); return fail(ION_E_NOMEM, "batch tables"); }
        b->allocs.push_back(*p);
        return ION_OK;
    };
    std::vector<DevLbm> views(count);
    std::vector<uint32_t> bins(count + 1, 0);
    for (uint32_t i = 0; i < count; i++) {
        views[i] = domains[i]->L;
        bins[i + 1] = bins[i] + (b->mhd ? domains[i]->L.n_lod_own : 0u);
    }
    b->total_bins = bins[count];
    int rc = dalloc((void**)&b->d_doms, sizeof(DevLbm) * count);
    if (!rc) rc = dalloc((void**)&b->d_bin_off, sizeof(uint32_t) * (count + 1));
    if (!rc) rc = dalloc((void**)&b->d_sync, sizeof(uint32_t) * 4);
    for (int s = 0; s < 2 && !rc; s++) {
        std::vector<uint32_t> tiles(count + 1, 0);
        const uint32_t per = kBatchBlocks[s] * EB_CPT;  // cells per tile
        for (uint32_t i = 0; i < count; i++) tiles[i + 1] = tiles[i] + (domains[i]->L.n + per - 1) / per;
        b->total_tiles[s] = tiles[count];
        rc = dalloc((void**)&b->d_tile_off[s], sizeof(uint32_t) * (count + 1));
        if (!rc && cudaMemcpy(b->d_tile_off[s], tiles.data(), sizeof(uint32_t) * (count + 1), cudaMemcpyHostToDevice) != cudaSuccess)
            rc = fail(ION_E_CUDA, "batch table upload");
        std::vector<uint32_t> bricks(count + 1, 0);
        for (uint32_t i = 0; i < count; i++) {
            const DevLbm& L = domains[i]->L;
            bricks[i + 1] = bricks[i] + eb_bricks(L.nx, L.ny, L.nz) * (256u / kBatchBlocks[s]);
        }
        b->total_bricks[s] = bricks[count];
        if (!rc) rc = dalloc((void**)&b->d_brick_off[s], sizeof(uint32_t) * (count + 1));
        if (!rc && cudaMemcpy(b->d_brick_off[s], bricks.data(), sizeof(uint32_t) * (count + 1), cudaMemcpyHostToDevice) != cudaSuccess)
            rc = fail(ION_E_CUDA, "batch table upload");
    }
    // the row-staged stencil when every domain's rows are whole 16-byte streams of at most
    // BATCH_ROW_MAX cells and its slot offsets fit in 32 bits (as for k_sc_rows_ws)
    bool rows_ok = true;
    std::vector<uint32_t> rows(count + 1, 0);
    for (uint32_t i = 0; i < count; i++) {
        const DevLbm& L = domains[i]->L;
        rows_ok = rows_ok && L.nx % 16u == 0u && L.nx <= BATCH_ROW_MAX && 19ull * L.n < (1ull << 32);
        rows[i + 1] = rows[i] + L.ny * L.nz;
    }
    if (!rc && rows_ok) {
        b->total_rows = rows[count];
        rc = dalloc((void**)&b->d_row_off, sizeof(uint32_t) * (count + 1));
        if (!rc && cudaMemcpy(b->d_row_off, rows.data(), sizeof(uint32_t) * (count + 1), cudaMemcpyHostToDevice) != cudaSuccess)
            rc = fail(ION_E_CUDA, "batch table upload");
    }
    if (!rc && (cudaMemcpy(b->d_doms, views.data(), sizeof(DevLbm) * count, cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemcpy(b->d_bin_off, bins.data(), sizeof(uint32_t) * (count + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemset(b->d_sync, 0, sizeof(uint32_t) * 4) != cudaSuccess))
        rc = fail(ION_E_CUDA, "batch table upload");
    if (rc) { destroy_batch(b); return rc; }
    for (auto& e : b->ev) cudaEventCreate(&e);
    *out = b;
    return ION_OK;
}

int ion_batch_destroy(ion_batch* b) {
    destroy_batch(b);
    return ION_OK;
}

// Autotuner: on the first run every launch shape (threads per block x blocks
// per SM that fit on the SM) advances the batch by two real steps, timed with
// CUDA events; the fastest shape is kept.  Results do not depend on the shape,
// so the tuning steps are ordinary steps of the simulation.
static int batch_autotune(ion_batch* b, uint64_t& steps) {
    float best = 1e30f;
    for (uint32_t block : kBatchBlocks) {
        const int maxb = batch_max_blocks_per_sm(b->ft, b->mhd, b->fast, b->total_rows > 0u, (int)block);
        for (int bps = 1; bps <= std::min(maxb, 4); bps++) {
            if (steps < 2) break;
            const uint32_t grid = (uint32_t)(bps * b->sms);
            CK(cudaEventRecord(b->ev[0], b->stream));
            int rc = batch_launch(b, block, grid);
            if (!rc) rc = batch_launch(b, block, grid);
            if (rc) return rc;
            CK(cudaEventRecord(b->ev[1], b->stream));
            CK(cudaEventSynchronize(b->ev[1]));
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]));
            steps -= 2;
            b->tuning.push_back({(float)block, (float)grid, ms / 2.0f});
            if (ms < best) { best = ms; b->block = block; b->grid = grid; }
        }
    }
    if (b->grid == 0) {  // not enough steps to tune: the middle shape
        b->block = 256;
        b->grid = (uint32_t)(std::max(1, std::min(2, batch_max_blocks_per_sm(b->ft, b->mhd, b->fast, b->total_rows > 0u, 256))) *
                             b->sms);
    } else {
        b->tuned = true;
    }
    return ION_OK;
}

int ion_batch_run(ion_batch* b, uint64_t steps) {
    if (!b) return fail(ION_E_INVALID, "null batch");
    const uint64_t total = steps;
    if (!b->tuned) {
        int rc = batch_autotune(b, steps);
        if (rc) return rc;
    }
    if ((b->t & 1u) && steps) {
        int rc = batch_launch(b, b->block, b->grid);
        if (rc) return rc;
        steps--;
    }
    if (steps >= 4 && !b->graph && !b->graph_failed) {
        cudaGraph_t g;
        bool ok = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            const uint64_t t0 = b->t;
            const cudaError_t e1 = launch_batch_step(batch_view(b, b->block), b->ft, b->mhd, b->fast, b->grid, b->block, 0, b->stream);
            const cudaError_t e2 = launch_batch_step(batch_view(b, b->block), b->ft, b->mhd, b->fast, b->grid, b->block, 1, b->stream);
            const cudaError_t e3 = cudaStreamEndCapture(b->stream, &g);
            b->t = t0;
            ok = e1 == cudaSuccess && e2 == cudaSuccess && e3 == cudaSuccess &&
                 cudaGraphInstantiate(&b->graph, g, 0) == cudaSuccess;
            if (e3 == cudaSuccess) cudaGraphDestroy(g);
        }
        if (!ok) { b->graph = nullptr; b->graph_failed = true; cudaGetLastError(); }
    }
    if (b->graph) {
        for (; steps >= 2; steps -= 2) {
            CK(cudaGraphLaunch(b->graph, b->stream));
            g_launches += b->mhd ? 4 : 2;
            b->t += 2;
        }
    }
    for (; steps > 0; steps--) {
        int rc = batch_launch(b, b->block, b->grid);
        if (rc) return rc;
    }
    for (ion_lbm* h : b->doms) h->t += total;
    return ION_OK;
}

int ion_batch_set_wait_limits(ion_batch* b, uint32_t barrier_polls, uint32_t tile_polls) {
    if (!b) return fail(ION_E_INVALID, "null batch");
    CK(cudaStreamSynchronize(b->stream));
    b->barrier_limit = barrier_polls;
    std::vector<DevLbm> views(b->doms.size());
    for (size_t i = 0; i < b->doms.size(); i++) {
        b->doms[i]->L.wait_limit = tile_polls;
        b->doms[i]->graph_dirty = true;
        views[i] = b->doms[i]->L;
    }
    CK(cudaMemcpy(b->d_doms, views.data(), sizeof(DevLbm) * views.size(), cudaMemcpyHostToDevice));
    if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }  // holds the old barrier limit
    b->graph_failed = false;
    return ION_OK;
}

int ion_batch_finish(ion_batch* b, int timeout_ms) {
    if (!b) return fail(ION_E_INVALID, "null batch");
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const cudaError_t e = cudaStreamQuery(b->stream);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) return fail(ION_E_CUDA, "batch stream: %s", cudaGetErrorString(e));
        if (timeout_ms >= 0 && std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(timeout_ms))
            return fail(ION_E_TIMEOUT, "batch still busy after %d ms", timeout_ms);
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    uint32_t err = 0;
    CK(cudaMemcpy(&err, b->d_sync + 2, 4, cudaMemcpyDeviceToHost));
    if (err) {
        cudaMemset(b->d_sync, 0, 4 * sizeof(uint32_t));
        return fail(ION_E_TIMEOUT, err == 2 ? "batch grid barrier timed out" : "batch field tile did not arrive in time");
    }
    return ION_OK;
}

int ion_batch_tuning(ion_batch* b, uint32_t i, uint32_t* block, uint32_t* grid, float* ms_per_step) {
    if (!b) return fail(ION_E_INVALID, "null batch");
    if (i == 0xFFFFFFFFu) {  // the chosen shape
        if (block) *block = b->block;
        if (grid) *grid = b->grid;
        if (ms_per_step) *ms_per_step = 0.0f;
        return b->tuned ? ION_OK : fail(ION_E_STATE, "not tuned yet");
    }
    if (i >= b->tuning.size()) return fail(ION_E_INVALID, "no tuning entry %u", i);
    if (block) *block = (uint32_t)b->tuning[i][0];
    if (grid) *grid = (uint32_t)b->tuning[i][1];
    if (ms_per_step) *ms_per_step = b->tuning[i][2];
    return ION_OK;
}

int ion_batch_record_event(ion_batch* b, int slot) {
    if (!b || slot < 0 || slot >= 4) return fail(ION_E_INVALID, "bad event slot");
    CK(cudaEventRecord(b->ev[slot], b->stream));
    return ION_OK;
}

int ion_batch_event_elapsed(ion_batch* b, int a, int c, float* ms) {
    if (!b || !ms || a < 0 || a >= 4 || c < 0 || c >= 4) return fail(ION_E_INVALID, "bad event slot");
    CK(cudaEventSynchronize(b->ev[c]));
    CK(cudaEventElapsedTime(ms, b->ev[a], b->ev[c]));
    return ION_OK;
}

// ---- learned far field ------------------------------------------------------------
static int ensure_surrogate(ion_lbm* h) {
    if (!h->cfg.ext_magneto_hydro) return fail(ION_E_STATE, "the learned far field needs ext_magneto_hydro");
    const uint32_t big = 1u << h->L.nd;
    if (h->L.depth < 2 || h->L.nx / big > 1 || h->L.ny / big > 1 || h->L.nz / big > 1)
        return fail(ION_E_CONFIG, "the learned far field needs LOD depth >= 2 and an empty reference near field");
    if (h->L.bsx > (uint32_t)ion::Surrogate::MAX_BLOCK)
        return fail(ION_E_CONFIG, "the learned far field needs LOD blocks of at most %d cells along x",
                    ion::Surrogate::MAX_BLOCK);
    if (h->sur) return ION_OK;
    h->sur.reset(new ion::Surrogate());
    const int rc = h->sur->init((int)h->L.nd, (float)h->L.bsx, (float)h->L.bsy, (float)h->L.bsz, (int)h->L.first_src);
    if (rc) { h->sur.reset(); return fail(rc, "surrogate buffers"); }
    return ION_OK;
}

int ion_lbm_surrogate_train(ion_lbm* h, uint32_t samples, uint32_t epochs, uint32_t batch, float lr, uint64_t seed,
                            float* rel_err) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    if (samples < 2 || batch == 0 || batch > samples) return fail(ION_E_INVALID, "bad sample/batch counts");
    int rc = ensure_surrogate(h);
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->stream));
    rc = h->sur->train((int)samples, (int)epochs, (int)batch, lr, seed, h->stream, rel_err);
    if (rc) return fail(rc, "surrogate training failed");
    h->graph_dirty = true;
    return ION_OK;
}

int ion_lbm_surrogate_info(ion_lbm* h, float* rel_err_fp32, float* rel_err_bf16, float* loss, uint32_t loss_cap,
                           uint32_t* epochs) {
    if (!h || !h->sur) return fail(ION_E_STATE, "no surrogate");
    if (rel_err_fp32) *rel_err_fp32 = h->sur->rel32();
    if (rel_err_bf16) *rel_err_bf16 = h->sur->rel16();
    const auto& L = h->sur->loss_history();
    if (epochs) *epochs = (uint32_t)L.size();
    for (uint32_t i = 0; loss && i < loss_cap && i < L.size(); i++) loss[i] = L[i];
    return ION_OK;
}

int ion_lbm_surrogate_save(ion_lbm* h, const char* path) {
    if (!h || !path) return fail(ION_E_INVALID, "null argument");
    if (!h->sur || !h->sur->ready()) return fail(ION_E_STATE, "no trained surrogate");
    const int rc = h->sur->save(path);
    return rc ? fail(rc, "cannot write \"%s\"", path) : ION_OK;
}

int ion_lbm_surrogate_load(ion_lbm* h, const char* path) {
    if (!h || !path) return fail(ION_E_INVALID, "null argument");
    int rc = ensure_surrogate(h);
    if (rc) return rc;
    rc = h->sur->load(path, h->stream);
    if (rc) return fail(rc, "cannot read a surrogate for this grid from \"%s\"", path);
    h->graph_dirty = true;
    return ION_OK;
}

int ion_lbm_surrogate_configure(ion_lbm* h, float tolerance, uint32_t check_cells) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    int rc = ensure_surrogate(h);
    if (rc) return rc;
    if (!(tolerance >= 0.0f) || check_cells == 0) return fail(ION_E_INVALID, "bad tolerance or sample count");
    h->sur->configure(tolerance, check_cells, h->stream);
    CKL();
    h->graph_dirty = true;
    return ION_OK;
}

int ion_lbm_surrogate_stats(ion_lbm* h, uint64_t* checks, uint64_t* fallbacks, uint64_t* nonfinite, float* err_e,
                            float* err_b) {
    if (!h || !h->sur) return fail(ION_E_STATE, "no surrogate");
    unsigned long long* c;
    float* last;
    h->sur->stats_device(&c, &last);
    unsigned long long hc[3] = {0, 0, 0};
    float hl[2] = {0, 0};
    CK(cudaMemcpyAsync(hc, c, sizeof hc, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(hl, last, sizeof hl, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (checks) *checks = hc[0];
    if (fallbacks) *fallbacks = hc[1];
    if (nonfinite) *nonfinite = hc[2];
    if (err_e) *err_e = hl[0];
    if (err_b) *err_b = hl[1];
    return ION_OK;
}

int ion_lbm_surrogate_weights(ion_lbm* h, float* out, const float* in, size_t count) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    int rc = ensure_surrogate(h);
    if (rc) return rc;
    if (count != h->sur->weight_count())
        return fail(ION_E_INVALID, "the network has %zu weights, got %zu", h->sur->weight_count(), count);
    if (out) { rc = h->sur->get_weights(out); if (rc) return fail(rc, "weights"); }
    if (in) { rc = h->sur->set_weights(in, h->stream); if (rc) return fail(rc, "weights"); h->graph_dirty = true; }
    return ION_OK;
}

int ion_lbm_surrogate_grad(ion_lbm* h, const float* x, const float* t, uint32_t batch, float* loss, float* grad) {
    if (!h || !x || !t || !loss || !grad || batch == 0) return fail(ION_E_INVALID, "null argument");
    int rc = ensure_surrogate(h);
    if (rc) return rc;
    rc = h->sur->grad(x, t, (int)batch, loss, grad, h->stream);
    return rc ? fail(rc, "surrogate gradient") : ION_OK;
}

int ion_lbm_surrogate_targets(ion_lbm* h, const float* x, float* t, uint32_t samples, float* scale_e, float* scale_b) {
    if (!h || !x || !t || samples == 0) return fail(ION_E_INVALID, "null argument");
    int rc = ensure_surrogate(h);
    if (rc) return rc;
    rc = h->sur->targets(x, t, (int)samples, h->stream);
    if (rc) return fail(rc, "surrogate targets");
    if (scale_e) *scale_e = h->sur->out_scale_e();
    if (scale_b) *scale_b = h->sur->out_scale_b();
    return ION_OK;
}

int ion_lbm_surrogate_forward(ion_lbm* h, const float* x, float* y, int bf16) {
    if (!h || !x || !y) return fail(ION_E_INVALID, "null argument");
    int rc = ensure_surrogate(h);
    if (rc) return rc;
    rc = h->sur->forward(x, y, bf16 != 0, h->stream);
    return rc ? fail(rc, "surrogate forward") : ION_OK;
}

int ion_lbm_set_field_mode(ion_lbm* h, int mode) {
    if (!h) return fail(ION_E_INVALID, "null handle");
    if (!h->cfg.ext_magneto_hydro) return fail(ION_E_STATE, "field modes apply to ext_magneto_hydro");
    if (mode < ION_FIELD_BITWISE || mode > ION_FIELD_SURROGATE) return fail(ION_E_INVALID, "unknown field mode %d", mode);
    if (mode == ION_FIELD_SURROGATE) {
        int rc = ensure_surrogate(h);
        if (rc) return rc;
    }
    h->cfg.field_mode = (uint8_t)mode;
    h->graph_dirty = true;
    return ION_OK;
}

// ---- device selection and the FP32 peak probe ---------------------------------
int ion_select_device(int device) {
    CK(cudaSetDevice(device));
    return ION_OK;
}

int ion_probe_fp32_peak(double* tflops) {
    if (!tflops) return fail(ION_E_INVALID, "null argument");
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    float* out = nullptr;
    CK(cudaMalloc(&out, 1024 * sizeof(float)));
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int blocks = sms * 8, iters = 1 << 16;
    launch_fma_probe(out, blocks, 1024, 0);  // warm-up
    cudaEventRecord(a, 0);
    launch_fma_probe(out, blocks, iters, 0);
    cudaEventRecord(b, 0);
    g_launches += 2;
    cudaError_t e = cudaEventSynchronize(b);
    float ms = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess) return fail(ION_E_CUDA, "fma probe: %s", cudaGetErrorString(e));
    const double flops = 2.0 * 8.0 * (double)iters * 256.0 * (double)blocks;  // FMA = 2 FLOP
    *tflops = flops / (ms * 1e-3) / 1e12;
    return ION_OK;
}

int ion_check_shared_division(uint64_t samples, uint64_t seed, uint64_t* mismatches, float* first_bad) {
    if (!mismatches) return fail(ION_E_INVALID, "null argument");
    unsigned long long* d_bad = nullptr;
    float* d_first = nullptr;
    CK(cudaMalloc(&d_bad, sizeof(unsigned long long)));
    if (cudaMalloc(&d_first, 2 * sizeof(float)) != cudaSuccess) {
        cudaFree(d_bad);
        return fail(ION_E_NOMEM, "division check buffers");
    }
    cudaMemset(d_bad, 0, sizeof(unsigned long long));
    cudaMemset(d_first, 0, 2 * sizeof(float));
    launch_div_check(samples, seed, d_bad, d_first, 0);
    g_launches++;
    unsigned long long bad = 0;
    float first[2] = {0.0f, 0.0f};
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(&bad, d_bad, sizeof bad, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(first, d_first, sizeof first, cudaMemcpyDeviceToHost);
    cudaFree(d_bad);
    cudaFree(d_first);
    if (e != cudaSuccess) return fail(ION_E_CUDA, "division check: %s", cudaGetErrorString(e));
    *mismatches = bad;
    if (first_bad) { first_bad[0] = first[0]; first_bad[1] = first[1]; }
    return ION_OK;
}

int ion_check_tcgen05_conv(int nd, int cin, int cout, int dil, uint64_t seed, float* max_rel_err) {
    if (!max_rel_err) return fail(ION_E_INVALID, "null argument");
    const int rc = ion::conv_tc_selftest(nd, cin, cout, dil, seed, max_rel_err, 0);
    g_launches += 4;
    return rc ? fail(rc, "tcgen05 convolution self-test (nd %d, cin %d, cout %d)", nd, cin, cout) : ION_OK;
}

// ---- device codec check -------------------------------------------------------
int ion_codec_roundtrip(int float_type, const float* in, uint16_t* enc, float* dec, const uint16_t* raw, float* raw_dec,
                        uint64_t n) {
    if (float_type != ION_FP16S && float_type != ION_FP16C) return fail(ION_E_INVALID, "codec must be FP16S or FP16C");
    if (!n) return ION_OK;
    float *d_in = nullptr, *d_dec = nullptr, *d_rdec = nullptr;
    uint16_t *d_enc = nullptr, *d_raw = nullptr;
    int rc = ION_OK;
    if (cudaMalloc(&d_in, n * 4) != cudaSuccess || cudaMalloc(&d_dec, n * 4) != cudaSuccess ||
        cudaMalloc(&d_rdec, n * 4) != cudaSuccess || cudaMalloc(&d_enc, n * 2) != cudaSuccess ||
        cudaMalloc(&d_raw, n * 2) != cudaSuccess) {
        rc = fail(ION_E_NOMEM, "codec buffers");
    } else {
        cudaMemcpy(d_in, in, n * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(d_raw, raw, n * 2, cudaMemcpyHostToDevice);
        launch_codec(float_type, d_in, d_enc, d_dec, d_raw, d_rdec, n, 0);
        g_launches++;
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = fail(ION_E_CUDA, "codec kernel");
        cudaMemcpy(enc, d_enc, n * 2, cudaMemcpyDeviceToHost);
        cudaMemcpy(dec, d_dec, n * 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(raw_dec, d_rdec, n * 4, cudaMemcpyDeviceToHost);
    }
    cudaFree(d_in); cudaFree(d_dec); cudaFree(d_rdec); cudaFree(d_enc); cudaFree(d_raw);
    return rc;
}

}  // extern "C"
