/*
 * ionsolver.h -- C ABI of the GB300 (sm_103a) implementation of IonSolver's
 * single-node MHD lattice-Boltzmann timestep.
 *
 * Every entry point replaces one call of the reference's Rust API for this
 * path; the reference interface is cited beside each declaration as
 * `file:line` inside the IonSolver crate (src/...).  Conventions:
 *
 *   - every function returns int: ION_OK (0) or a negative ION_E_* code;
 *     ion_last_error() gives a message for the calling thread.  Nothing
 *     aborts the process (the reference panics or exits instead).
 *   - host arrays are caller-owned and copied; device memory is owned by the
 *     handle.  Arrays use the reference's SoA layout: a cell index is
 *     n = x + (y + z*n_y)*n_x, vectors are [3][N], DDFs are [q][N].
 *   - one handle owns one CUDA stream and is not thread-safe; distinct
 *     handles may be used from distinct threads.
 */
#ifndef IONSOLVER_H
#define IONSOLVER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ION_ABI_VERSION 2

/* ---- status codes ---------------------------------------------------- */
#define ION_OK 0
#define ION_E_INVALID   (-1)  /* bad argument / null pointer / wrong size   */
#define ION_E_CONFIG    (-2)  /* configuration not supported by this build  */
#define ION_E_CUDA      (-3)  /* CUDA runtime error                         */
#define ION_E_NOMEM     (-4)  /* device or host allocation failed           */
#define ION_E_IO        (-5)  /* file could not be opened / written         */
#define ION_E_FORMAT    (-6)  /* file content malformed (header, size, ...) */
#define ION_E_TIMEOUT   (-7)  /* bounded wait expired                       */
#define ION_E_STATE     (-8)  /* call not valid in the handle's state       */

/* ---- enums (values equal the reference's `as u8` casts) -------------- */
/* VelocitySet, src/lbm/types.rs:16-26 */
enum { ION_D2Q9 = 0, ION_D3Q15 = 1, ION_D3Q19 = 2, ION_D3Q27 = 3 };
/* RelaxationTime, src/lbm/types.rs:55-61 */
enum { ION_SRT = 0, ION_TRT = 1 };
/* FloatType, src/lbm/types.rs:75-83 */
enum { ION_FP16S = 0, ION_FP16C = 1, ION_FP32 = 2 };
/* Propellant, src/lbm/units.rs:214-222 */
enum { ION_PROP_H = 0, ION_PROP_HE, ION_PROP_NE, ION_PROP_AR, ION_PROP_KR, ION_PROP_XE };
/* How the dynamic E/B far field is evaluated each step (no reference
 * counterpart: the reference always runs update_e_b_dynamic,
 * src/kernels/sim_kernels.cl:897-993).
 *   BITWISE: the reference's summation order and IEEE operations, results
 *            bit-identical to the reference kernel run in cell order;
 *   FAST:    same sources and sum order, reciprocal-sqrt/FMA arithmetic;
 *   SURROGATE: learned far field with a sampled exact check and fallback. */
enum { ION_FIELD_BITWISE = 0, ION_FIELD_FAST = 1, ION_FIELD_SURROGATE = 2 };

/* Field identifiers for read/write (the pub buffers of LbmDomain,
 * src/lbm/domain.rs:45-74). */
enum {
    ION_FIELD_FI = 0,      /* DDFs, [q][N], f32 or u16 (float_type)        */
    ION_FIELD_RHO = 1,     /* f32 [N]                                      */
    ION_FIELD_U = 2,       /* f32 [3][N]                                   */
    ION_FIELD_FLAGS = 3,   /* u8  [N]                                      */
    ION_FIELD_F = 4,       /* f32 [3][N] force field (ext_force_field)     */
    ION_FIELD_E_STAT = 5,  /* f32 [3][N]                                   */
    ION_FIELD_B_STAT = 6,  /* f32 [3][N]                                   */
    ION_FIELD_E_DYN = 7,   /* f32 [3][N] (or larger, see ion_lbm_field_info)*/
    ION_FIELD_B_DYN = 8,   /* f32 [3][N]                                   */
    ION_FIELD_FQI = 9,     /* charge DDFs, [7][N], f32 or u16              */
    ION_FIELD_EI = 10,     /* electron-gas DDFs, [q][N], f32 or u16        */
    ION_FIELD_Q = 11,      /* f32 [N] cell charge                          */
    ION_FIELD_QU_LOD = 12, /* f32 [n_lod][4] charge + velocity LOD         */
    ION_FIELD_E_VAR = 13,  /* f32 [3][N] oscillating field (ext_subgrid_ecr) */
    ION_FIELD_ETI = 14,    /* electron-temperature DDFs, [7][N], f32 or u16 */
    ION_FIELD_ET = 15,     /* f32 [N] electron temperature                 */
    ION_FIELD_COUNT = 16
};

/* ModelType -> flag byte, src/mesh.rs:9-14, 309-314 */
enum { ION_MODEL_SOLID = 0, ION_MODEL_MAGNET = 1, ION_MODEL_CHARGED = 2, ION_MODEL_CHARGED_ECR = 3 };

/* Units, src/lbm/units.rs:14-27 */
typedef struct ion_units {
    float m, kg, s, a, k;
    int32_t prop;
} ion_units;

/* LbmConfig, src/lbm/mod.rs:45-101.  The graphics_config member is replaced
 * by `update_fields`, its only effect on the timestep (graphics_active turns
 * on UPDATE_FIELDS, src/lbm/domain.rs:856); `field_mode` is new. */
typedef struct ion_config {
    int32_t velocity_set;          /* ION_D2Q9 ... ION_D3Q27   */
    int32_t relaxation_time;       /* ION_SRT / ION_TRT        */
    int32_t float_type;            /* ION_FP16S/ION_FP16C/ION_FP32 */
    ion_units units;
    uint32_t n_x, n_y, n_z;
    uint32_t d_x, d_y, d_z;        /* must be 1: one GPU, no decomposition */
    float nu;
    float f_x, f_y, f_z;
    uint8_t ext_equilibrium_boundaries;
    uint8_t ext_volume_force;
    uint8_t ext_force_field;
    uint8_t ext_magneto_hydro;
    uint8_t ext_subgrid_ecr;       /* needs ext_magneto_hydro  */
    uint8_t mhd_lod_depth;
    uint8_t update_fields;
    uint8_t field_mode;            /* ION_FIELD_*              */
    float ecr_freq, ecr_field_strength;
    uint64_t run_steps;
} ion_config;

/* Constants derived from Units that the kernels use
 * (src/lbm/units.rs:149-197; src/lbm/domain.rs:808, 838-848). */
typedef struct ion_constants {
    float w;        /* DEF_W   = 1/(3 nu + 1/2)            */
    float ke;       /* DEF_KE  = ke_lu                     */
    float kmu;      /* DEF_KMU = mu_0_lu / (4 pi)          */
    float kmu0;     /* DEF_KMU0 = mu_0_lu                  */
    float kkge;     /* DEF_KKGE = kkge_lu                  */
    float kimg;     /* DEF_KIMG = kimg_lu                  */
    float kvev;     /* DEF_KVEV = kveV_lu                  */
    float kme;      /* DEF_KME  = kme_lu                   */
    float wq;       /* DEF_WQ  = 1/(2 k_charge_expansion + 1/2) */
    float epsilon_0;/* epsilon_0_lu                        */
    float mu_0;     /* mu_0_lu                             */
    float kkbme;    /* DEF_KKBME = kkBme_lu (SUBGRID_ECR)  */
    float keabs;    /* DEF_KEABS = keabs_lu (SUBGRID_ECR)  */
} ion_constants;

typedef struct ion_lbm ion_lbm;   /* opaque: Lbm with its single LbmDomain */

/* ---- library ---------------------------------------------------------- */
int ion_abi_version(void);
/* cudaSetDevice for the calling thread (the reference picks devices in
 * opencl::device_selection, src/opencl.rs:9-63); handles use the device that
 * is current when they are created. */
int ion_select_device(int device);
/* Measured FP32 FMA throughput of the current device in TFLOP/s (FMA = 2
 * FLOP; no reference counterpart): the roofline denominator of the
 * FP32-bound field kernel. */
int ion_probe_fp32_peak(double* tflops);
const char* ion_last_error(void);
/* Number of CUDA kernel launches this process made through the library. */
uint64_t ion_kernel_launch_count(void);

/* LbmConfig::new(), src/lbm/mod.rs:105-135 */
int ion_config_default(ion_config* cfg);
/* Units::new(), src/lbm/units.rs:30-39 */
int ion_units_default(ion_units* u);
/* Units::set(...), src/lbm/units.rs:41-60 */
int ion_units_set(ion_units* u, float lbm_length, float lbm_velocity, float lbm_rho,
                  float lbm_charge, float lbm_temp, float si_length, float si_velocity,
                  float si_rho, float si_charge, float si_temp);
/* The kernel constants for a config (get_device_defines, src/lbm/domain.rs:736-858) */
int ion_constants_from_config(const ion_config* cfg, ion_constants* out);
/* Units::nu_si_lu / magnetization_si_lu / charge_si_lu / len_si_lu
 * (src/lbm/units.rs:126-128, 145-147, 130-133, 102-104): what selects the conversion:
 * 0 = nu, 1 = magnetization, 2 = charge, 3 = length. */
int ion_units_si_to_lu(const ion_units* u, int what, float value, float* out);

/* ---- lifecycle (Lbm::new, src/lbm/mod.rs:166-210; LbmDomain::new,
 *      src/lbm/domain.rs:88-409) ------------------------------------------ */
int ion_lbm_create(const ion_config* cfg, ion_lbm** out);
int ion_lbm_destroy(ion_lbm* h);
int ion_lbm_get_config(const ion_lbm* h, ion_config* out);

/* ---- step loop -------------------------------------------------------- */
/* Lbm::initialize, src/lbm/mod.rs:214-231 */
int ion_lbm_initialize(ion_lbm* h);
/* Finite-plasma start (no reference counterpart; MHD handles only): the next
 * ion_lbm_initialize starts the electron gas at density rho_e0 instead of 0
 * (src/kernels/sim_kernels.cl:823) and the charge lattice at Q + rho_e0
 * instead of Q (sim_kernels.cl:818), so the net charge Q = rho_q - rho_e is
 * unchanged.  The reference's electron gas starts empty, and its velocity
 * j/rho_e turns 0/0 within a few steps (sim_kernels.cl:230-232), after which
 * every MHD field is NaN; a background keeps the state finite.  rho_e0 = 0
 * (the default) is the reference's start. */
int ion_lbm_set_electron_background(ion_lbm* h, float rho_e0);
/* Lbm::do_time_step, src/lbm/mod.rs:250-272 (asynchronous on the handle's
 * stream; the reference blocks in finish_queues, mod.rs:267-270) */
int ion_lbm_do_time_step(ion_lbm* h);
/* Lbm::run, src/lbm/mod.rs:235-245 (initializes first if needed; replays
 * the step as a captured CUDA graph; asynchronous) */
int ion_lbm_run(ion_lbm* h, uint64_t steps);
/* Lbm::get_time_step, src/lbm/mod.rs:492-494 */
int ion_lbm_get_time_step(const ion_lbm* h, uint64_t* t);
/* Lbm::finish_queues, src/lbm/mod.rs:275-279, with a bound on the wait:
 * returns ION_E_TIMEOUT if the stream is still busy after timeout_ms
 * (timeout_ms < 0: wait without bound). */
int ion_lbm_finish_queues(ion_lbm* h, int timeout_ms);
/* Bounded device waits (no reference counterpart; the reference's OpenCL
 * kernels do not wait on each other).  The row-staged stream_collide and the
 * E/B update wait for data they staged with bulk copies; a wait gives up after
 * `polls` polls, records the failure, lets its copies in flight land and skips
 * the rest of the launch, and ion_lbm_finish_queues then returns ION_E_TIMEOUT.
 * Default ION_WAIT_LIMIT_DEFAULT; 0 gives up at the first wait (used to test
 * the timeout path).  The skipped work leaves the state incomplete: initialize
 * again after a timeout. */
#define ION_WAIT_LIMIT_DEFAULT 16777216u
int ion_lbm_set_wait_limit(ion_lbm* h, uint32_t polls);
/* LbmDomain::enqueue_update_fields, src/lbm/domain.rs:432-441 */
int ion_lbm_update_fields(ion_lbm* h);

/* ---- field access (bwrite!/bread! on the pub buffers, e.g.
 *      src/setup.rs:180-184, src/file.rs:118-153, 233-269) --------------- */
/* element size in bytes and element count of a field (0 if absent) */
int ion_lbm_field_info(const ion_lbm* h, int field, size_t* elem_bytes, size_t* count);
int ion_lbm_write_field(ion_lbm* h, int field, const void* host, size_t bytes);
int ion_lbm_read_field(ion_lbm* h, int field, void* host, size_t bytes);
/* device pointer of a field (valid until ion_lbm_destroy) */
int ion_lbm_field_device_ptr(ion_lbm* h, int field, void** dptr, size_t* bytes);
/* the handle's cudaStream_t */
int ion_lbm_stream(ion_lbm* h, void** stream);

/* ---- geometry (Lbm::import_mesh*, voxelise_mesh, precompute_B/E;
 *      src/mesh.rs:233-343, src/lbm/mod.rs:284-314) ----------------------- */
/* Adds a triangle mesh given in lattice coordinates; p0/p1/p2 are [ntri][3].
 * The bounding box is computed as Mesh::update_bounds (src/mesh.rs:94-109). */
int ion_lbm_add_mesh(ion_lbm* h, const float* p0, const float* p1, const float* p2,
                     uint32_t ntri, uint32_t* index);
/* Lbm::import_mesh, src/mesh.rs:233-239 (binary STL) */
int ion_lbm_import_mesh(ion_lbm* h, const char* path, float scale, float ox, float oy, float oz,
                        float rx, float ry, float rz, uint32_t* index);
/* Lbm::import_mesh_reposition, src/mesh.rs:248-253 */
int ion_lbm_import_mesh_reposition(ion_lbm* h, const char* path, float cx, float cy, float cz,
                                   float rx, float ry, float rz, float size, uint32_t* index);
/* Mesh::translate, src/mesh.rs:121-130 */
int ion_lbm_mesh_translate(ion_lbm* h, uint32_t index, float dx, float dy, float dz);
/* a mesh's vertices, [ntri][3] each (the p0/p1/p2 arrays of Mesh,
 * src/mesh.rs:71-79); with p0 = p1 = p2 = NULL only *ntri is set */
int ion_lbm_mesh_triangles(const ion_lbm* h, uint32_t index, float* p0, float* p1, float* p2, uint32_t capacity,
                           uint32_t* ntri);
/* mesh bounds: out[0..2] = p_min, out[3..5] = p_max, out[6..8] = center */
int ion_lbm_mesh_bounds(const ion_lbm* h, uint32_t index, float* out9);
/* Lbm::voxelise_mesh(index, ModelType), src/mesh.rs:256-343.
 * v0..v2 = magnetization (A/m, Magnet) or v0 = charge (C, Charged*). */
int ion_lbm_voxelise_mesh(ion_lbm* h, uint32_t index, int model_type, float v0, float v1, float v2);
/* Lbm::precompute_B, src/lbm/mod.rs:284-297 */
int ion_lbm_precompute_b(ion_lbm* h);
/* Lbm::precompute_E, src/lbm/mod.rs:302-314 (static E of charged solids) */
int ion_lbm_precompute_e(ion_lbm* h);
/* Lbm::precompute_E_ECR (src/lbm/mod.rs:319-331): the field of ChargedECR /
 * Charged cells into E_var, the oscillating field of the SUBGRID_ECR extension */
int ion_lbm_precompute_e_ecr(ion_lbm* h);

/* ---- FP64 domain reductions (no reference counterpart) ----------------- */
/* Total mass and total charge in double: the sums of every stored DDF slot of
 * the gas lattice (mass) and of the charge lattice minus the electron gas
 * (charge), decoded from their storage type and accumulated in FP64, plus the
 * DDF shift (1 per cell and lattice).  Every slot counts, solid cells'
 * included: what streams into a wall slot comes back out of it. */
int ion_lbm_mass_charge(ion_lbm* h, double* mass, double* charge);

/* ---- persistence (file::write / file::read, src/file.rs:12-30, 42-306;
 *      FILE_LAYOUT.txt) --------------------------------------------------- */
int ion_lbm_save(ion_lbm* h, const char* path);
/* Creates a handle from an .ion file; cfg_inout supplies the fields the file
 * does not hold (as the reference's `config` argument does) and receives
 * the decoded config. */
int ion_lbm_load(const char* path, ion_config* cfg_inout, ion_lbm** out);

/* ---- timing helpers on the handle's stream ---------------------------- */
/* records a CUDA event on the handle's stream; slot 0..7 */
int ion_lbm_record_event(ion_lbm* h, int slot);
/* elapsed ms between two recorded slots (synchronizes on `end`) */
int ion_lbm_event_elapsed(ion_lbm* h, int start, int end, float* ms);
/* per-kernel timing: when enabled, every launch of the dominant kernels is
 * bracketed by events; read back as total ms and launch count per kernel. */
int ion_lbm_set_kernel_timing(ion_lbm* h, int enable);
/* kernel: 0 = stream_collide, 1 = update_e_b, 2 = lod bins */
int ion_lbm_kernel_time(ion_lbm* h, int kernel, double* total_ms, uint64_t* launches);
int ion_lbm_reset_kernel_time(ion_lbm* h);

/* ---- LbmConfig as JSON (file::read_config / file::write_config,
 *      src/file.rs:310-334; serde's layout of LbmConfig, src/lbm/mod.rs:45-101).
 *      Reading maps graphics_config.graphics_active to update_fields and
 *      ignores the other graphics settings; writing emits GraphicsConfig::new()
 *      with graphics_active = update_fields, plus a "field_mode" key that the
 *      reference ignores.  No device is needed. ---------------------------- */
int ion_config_write_json(const char* path, const ion_config* cfg);
int ion_config_read_json(const char* path, ion_config* cfg);

/* ---- full checkpoint (no reference counterpart: the reference resumes a
 *      .ion file from equilibrium, src/file.rs:42-188).  The file is the .ion
 *      image of ion_lbm_save followed by an extension block ("IONX") with the
 *      time step and every device buffer the next step reads (DDFs of all
 *      lattices, E/B, LOD bins, force field), so a restored handle continues
 *      bit for bit.  ion_lbm_load reads such a file as a plain .ion file. --- */
int ion_lbm_checkpoint(ion_lbm* h, const char* path);
int ion_lbm_restore(const char* path, ion_config* cfg, ion_lbm** out);

/* ---- learned far field (no reference counterpart; it stands in for the far
 *      part of update_e_b_dynamic, src/kernels/sim_kernels.cl:940-955).
 *      Per cell, LOD bins within Chebyshev distance 1 of the cell's own bin
 *      are summed exactly; the rest comes from a linear 3-D convolutional
 *      network on the LOD grid (4 channels in: q, q*v; 168 out: E and B at
 *      3 x 3 x 3 nodes of every block, 162 used), interpolated
 *      triquadratically.  Every step a
 *      sampled-cell check against the exact sum decides on the device whether
 *      the exact kernel recomputes the field.  Needs ext_magneto_hydro, LOD
 *      depth >= 2 and an empty reference near field. -------------------- */
/* Generates `samples` snapshots (random charge and current per bin, exact
 * far-field targets), trains with Adam on the GPU; rel_err = held-out
 * relative L2 error of the BF16 inference path. */
int ion_lbm_surrogate_train(ion_lbm* h, uint32_t samples, uint32_t epochs, uint32_t batch, float lr, uint64_t seed,
                            float* rel_err);
int ion_lbm_surrogate_info(ion_lbm* h, float* rel_err_fp32, float* rel_err_bf16, float* loss, uint32_t loss_cap,
                           uint32_t* epochs);
int ion_lbm_surrogate_save(ion_lbm* h, const char* path);
int ion_lbm_surrogate_load(ion_lbm* h, const char* path);
/* relative tolerance of the sampled check (default 1e-2) and cells per check
 * (default 1024); restarts the statistics and the sequence of sampled cells */
int ion_lbm_surrogate_configure(ion_lbm* h, float tolerance, uint32_t check_cells);
/* checks run, fallbacks taken, checks whose exact sample was non-finite, last
 * relative errors of E and B.  A component that is non-finite in both the
 * surrogate and the exact sum counts as agreeing: a non-finite source makes
 * the exact field non-finite everywhere, so the fallback cannot repair it. */
int ion_lbm_surrogate_stats(ion_lbm* h, uint64_t* checks, uint64_t* fallbacks, uint64_t* nonfinite, float* err_e,
                            float* err_b);
/* network weights (get into `out` and/or set from `in`; count = number of weights) */
int ion_lbm_surrogate_weights(ion_lbm* h, float* out, const float* in, size_t count);
/* mean squared error and its weight gradient for one batch: x [batch][4][V],
 * t [batch][168][V] (host, in the network's output scale) */
int ion_lbm_surrogate_grad(ion_lbm* h, const float* x, const float* t, uint32_t batch, float* loss, float* grad);
/* exact far-field targets t [samples][168][V] of sources x [samples][4][V]
 * (host), in field units; scale_e/scale_b: the network's output scales */
int ion_lbm_surrogate_targets(ion_lbm* h, const float* x, float* t, uint32_t samples, float* scale_e, float* scale_b);
/* one forward pass of x [4][V] into y [168][V] (host); bf16 != 0: tensor-core path */
int ion_lbm_surrogate_forward(ion_lbm* h, const float* x, float* y, int bf16);
/* switches the field mode of an MHD handle (ION_FIELD_*) */
int ion_lbm_set_field_mode(ion_lbm* h, int mode);

/* ---- batches of independent domains (no reference counterpart; the
 *      reference advances one domain per OpenCL queue, src/lbm/mod.rs:250-272)
 *      Every domain of a batch keeps its own buffers, size, units and flags;
 *      all must be D3Q19 with the same float type, MHD switch and field mode,
 *      at time steps of equal parity.  One cooperative launch per step
 *      advances all of them (stream_collide, LOD bins, E/B); results equal
 *      stepping each domain alone. ----------------------------------------- */
typedef struct ion_batch ion_batch;
int ion_batch_create(ion_lbm* const* domains, uint32_t count, ion_batch** out);
int ion_batch_destroy(ion_batch* b);
/* Advances every domain by `steps`.  The first call autotunes the launch
 * shape on its first steps (each candidate shape runs two real steps) and
 * then replays a CUDA graph of two steps. Asynchronous. */
int ion_batch_run(ion_batch* b, uint64_t steps);
/* bounded wait for the batch's stream; reports device-side timeouts */
int ion_batch_finish(ion_batch* b, int timeout_ms);
/* the batch step's poll limits: grid barrier between its phases (default
 * ION_BARRIER_LIMIT_DEFAULT, polls 64 ns apart) and staged-tile waits of every
 * domain (as ion_lbm_set_wait_limit); a wait that gives up ends the launch
 * and ion_batch_finish returns ION_E_TIMEOUT */
#define ION_BARRIER_LIMIT_DEFAULT 67108864u
int ion_batch_set_wait_limits(ion_batch* b, uint32_t barrier_polls, uint32_t tile_polls);
/* autotuner record i (block, grid, ms per step); i = 0xFFFFFFFF: the chosen shape */
int ion_batch_tuning(ion_batch* b, uint32_t i, uint32_t* block, uint32_t* grid, float* ms_per_step);
int ion_batch_record_event(ion_batch* b, int slot);
int ion_batch_event_elapsed(ion_batch* b, int start, int end, float* ms);

/* ---- FP64 sum without device allocation (no counterpart in the reference) --
 * Sum, in double precision, of `count` stored DDF values (decoded with
 * float_type) at device address d_values; the result is written to the
 * device double *d_sum, ordered on `stream` (a cudaStream_t, 0 = default).
 * For callers that cannot call cudaMalloc/cudaFree where they need the sum:
 * a host whose device memory is fully reserved by its own pool allocator, or
 * a stepping loop that must not take the implicit synchronisation of
 * cudaFree.  The scratch is a fixed 32 KiB array of partial sums in device
 * memory, held by every GPU that loads this library until the process exits.
 * At most ION_NOALLOC_MAX_VALUES values per call (else ION_E_INVALID).  The
 * first call on a device looks the array up with that device current; make
 * it before any stream capture.  All calls on a device share the array, so
 * calls that overlap on the GPU race; each call rewrites every partial it
 * reads, so nothing needs clearing between calls.  The looked-up address is
 * kept until the process exits: after cudaDeviceReset on a device, calls on
 * that device are not supported. */
#define ION_NOALLOC_MAX_VALUES 268435456ull
int ion_ddf_sum_f64_noalloc(const void* d_values, int float_type, uint64_t count, double* d_sum, void* stream);

/* ---- self-test of the BITWISE field's division (no reference counterpart):
 *      compares, bit for bit, the quotient formed from one correctly rounded
 *      reciprocal and two FMA corrections (used for the three divides by
 *      |R|^3 of sim_kernels.cl:931-935) with the IEEE division on `samples`
 *      pseudo-random operands in the ranges the E/B sums produce. ------- */
int ion_check_shared_division(uint64_t samples, uint64_t seed, uint64_t* mismatches, float* first_bad);

/* ---- self-test of the learned far field's tcgen05 convolution (no
 *      reference counterpart): the 3^3 convolution on pseudo-random BF16 data
 *      through tcgen05.mma (TMEM accumulator) against the mma.sync
 *      implementation; max |diff| / max |mma.sync result|.  nd^3 must be a
 *      multiple of 128; (cin, cout) in {(16, 32), (32, 32), (32, 168)}. ---- */
int ion_check_tcgen05_conv(int nd, int cin, int cout, int dil, uint64_t seed, float* max_rel_err);

/* ---- storage codecs on the device (no reference counterpart; exposes the
 *      FP16S/FP16C codecs of src/lbm/domain.rs:773-780 and
 *      src/kernels/sim_kernels.cl:79-90 for exhaustive checks) ------------ */
/* enc[i] = encode(in[i]), dec[i] = decode(enc[i]), raw_dec[i] = decode(raw[i]) */
int ion_codec_roundtrip(int float_type, const float* in, uint16_t* enc, float* dec, const uint16_t* raw,
                        float* raw_dec, uint64_t n);

#ifdef __cplusplus
}
#endif
#endif /* IONSOLVER_H */
