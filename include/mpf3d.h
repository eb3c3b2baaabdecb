/*
 * mpf3d.h -- C ABI of libmpf3d.so, the GB300 (sm_103a) implementation of the
 * 3D multi-phase-field step of daikihatanaka0327/multiphasefield-solidification-v2.
 *
 * Plain pointers, sizes and a stream handle; no C++ or framework types.  All
 * array pointers are DEVICE pointers unless a parameter says "host".  Every
 * function enqueues asynchronously on `stream` (a cudaStream_t passed as
 * void*, NULL = legacy default stream) and returns an MPF3D_* status code
 * describing argument validation and the launch; conditions found on the
 * device are OR-ed into the caller's optional `err` word (int32, device).
 *
 * Arrays use the reference's dense C-order layout:
 *   phi  [N][nx][ny][nz]   float32 or float64   (z fastest)
 *   mf   [depth][nx][ny][nz] int32,  nf [nx][ny][nz] int32
 *   temp [nx][ny][nz]      float32 or float64
 *   wij, aij, mij [N][N] float32,  n111 [N][8][3] float32
 */
#ifndef MPF3D_H
#define MPF3D_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* return codes */
#define MPF3D_OK 0
#define MPF3D_ERR_ARG (-1)    /* bad size, null pointer or unsupported combination */
#define MPF3D_ERR_DTYPE (-2)  /* dtype code not 0 (float32) or 1 (float64) */
#define MPF3D_ERR_CUDA (-3)   /* a CUDA call or launch failed */
#define MPF3D_ERR_TOO_LARGE (-4)

/* dtype codes */
#define MPF3D_F32 0
#define MPF3D_F64 1

/* bits OR-ed into the device `err` word */
#define MPF3D_DEV_MF_DEPTH 1      /* unchecked APT needed more rows than mf has */
#define MPF3D_DEV_NF_GT_KMAX 2    /* update met nf > KMAX (cell left untouched) */
#define MPF3D_DEV_BAD_ID 4        /* update met an mf id outside [0, N) */
#define MPF3D_DEV_SLOT_OVERFLOW 8 /* compact stepper: more phases than slots */
#define MPF3D_DEV_BAD_INPUT 16    /* compact conversion met a negative/NaN phi */
#define MPF3D_DEV_GEMM_ABORT 32   /* tcgen05 GEMM: a bounded wait ran out; the CTA's outputs are NaN */
#define MPF3D_DEV_STAGING_TIMEOUT 64 /* compact step: a TMA staging copy did not land in time (the block's
                                      * cells were not processed) */

/* compile-time bound on active phases per cell (reference KMAX) */
#define MPF3D_KMAX 50

/* The 13 floating-point kernel arguments of the reference's phase update, in
 * the reference's argument order; bit i of f32mask says argument i was a
 * float32 (np.float32) rather than a float64, which changes the arithmetic
 * type of several expressions exactly as in the reference. */
enum {
    MPF3D_S_DX = 0, MPF3D_S_DT, MPF3D_S_T_MELT, MPF3D_S_SF, MPF3D_S_EPS0_SL, MPF3D_S_W0_SL,
    MPF3D_S_A0, MPF3D_S_DELTA_A, MPF3D_S_MU_A, MPF3D_S_P_ROUND, MPF3D_S_G2_FLOOR, MPF3D_S_KSI,
    MPF3D_S_THETA_C_RAD, MPF3D_S_COUNT
};
typedef struct mpf3d_scalars {
    double v[MPF3D_S_COUNT];
    uint32_t f32mask;
} mpf3d_scalars;

/* ---- dense drop-in tier (reference numerics) ---------------------------- */

/* Replaces kernel_update_nfmf_3d (checked = 0) and
 * kernel_update_nfmf_3d_checked (checked = 1), src/gpu_kernels_3d.py:462-527.
 * status: int32[2] device array, required when checked ({overflow, max n},
 * atomic max as in the reference).  Unchecked writes are clamped to `depth`
 * rows and set MPF3D_DEV_MF_DEPTH instead of running past the array. */
int mpf3d_dense_apt(const void *phi, int phi_dtype, int N, int nx, int ny, int nz, int32_t *mf,
                    int depth, int32_t *nf, int32_t *status, int checked, int32_t *err,
                    void *stream);

/* Replaces kernel_update_phasefield_active_3d (switchable = 0) and
 * kernel_update_phasefield_active_3d_switchable (switchable = 1),
 * src/gpu_kernels_3d.py:530-830.  phi and phi_new share phi_dtype. */
int mpf3d_dense_update(const void *phi, void *phi_new, int phi_dtype, const void *temp,
                       int temp_dtype, const int32_t *mf, int depth, const int32_t *nf,
                       const float *wij, const float *aij, const float *mij, const float *n111,
                       int N, int nx, int ny, int nz, const mpf3d_scalars *scalars, int switchable,
                       int enable_anisotropy, int enable_torque, int32_t *err, void *stream);

/* Replaces kernel_update_temp_3d, src/gpu_kernels_3d.py:833-838:
 * temp -= cooling_rate (float32 arithmetic when both are float32). */
int mpf3d_dense_temp(void *temp, int temp_dtype, double cooling_rate, int rate_is_f32, int64_t n,
                     void *stream);

/* ---- dense 2D kernels (reference numerics) --------------------------------
 * The reference's 2D module src/gpu_kernels.py, on its dense [N][nx][ny]
 * arrays (x periodic, y mirror).  The reference's verification suite runs it
 * beside the 3D step (tests/verification_3d.py:21-25, 1509-1535). */

/* Replaces kernel_update_nfmf, src/gpu_kernels.py:337-358.  Writes past
 * `depth` rows are dropped and set MPF3D_DEV_MF_DEPTH. */
int mpf2d_dense_apt(const void *phi, int phi_dtype, int N, int nx, int ny, int32_t *mf, int depth,
                    int32_t *nf, int32_t *err, void *stream);

/* Replaces kernel_update_phasefield_active, src/gpu_kernels.py:361-517.
 * N >= 2: the reference's dominant-solid lookup defaults to grain 1. */
int mpf2d_dense_update(const void *phi, void *phi_new, int phi_dtype, const void *temp, int temp_dtype,
                       const int32_t *mf, int depth, const int32_t *nf, const float *wij,
                       const float *aij, const float *mij, const float *n111, int N, int nx, int ny,
                       const mpf3d_scalars *scalars, int32_t *err, void *stream);

/* Replaces kernel_update_temp, src/gpu_kernels.py:520-525. */
int mpf2d_dense_temp(void *temp, int temp_dtype, double cooling_rate, int rate_is_f32, int nx, int ny,
                     void *stream);

/* ---- compact FP32 tier (three-kernel step) -------------------------------
 * State of one buffer (x fastest: cell = (k*ny + m)*nx + l):
 *   head uint32[cells]        bits 0-6 number n of stored phases (phi > 0),
 *                             bit 7 single value stored explicitly,
 *                             bits 8-23 id of the smallest stored phase
 *   idx  uint16[slots][cells] ids of stored phases 1..n-1, ascending (slot 0 unused)
 *   val  float[slots][cells]  fractions of stored phases 0..n-1; a cell whose
 *                             only stored phase is exactly 1 keeps no value
 * slots is 4, 8 or 16.  No reference counterpart for the layout: it replaces
 * the dense phi [N][nx][ny][nz] + mf/nf arrays of src/gpu_kernels_3d.py. */

/* dense phi (z fastest, float32/float64) -> compact state.  Negative or NaN
 * entries set MPF3D_DEV_BAD_INPUT; more than `slots` positive phases in a
 * cell set MPF3D_DEV_SLOT_OVERFLOW. */
int mpf3d_compact_from_dense(const void *phi, int phi_dtype, int N, int nx, int ny, int nz, int slots,
                             uint32_t *head, uint16_t *idx, float *val, int32_t *err, void *stream);

/* Device address of page-locked (pinned) host memory, for the converters
 * below: with it mpf3d_compact_from_dense reads dense phi straight from
 * host memory and mpf3d_compact_to_dense writes it straight back, over the
 * CPU-GPU link, with no staging copy in device memory.  MPF3D_ERR_ARG when
 * `host` is not page-locked.  No reference counterpart (the reference copies
 * whole device arrays with cuda.to_device / copy_to_host). */
int mpf3d_host_device_pointer(const void *host, void **device);

/* compact state -> dense phi (every phase written, zeros included). */
int mpf3d_compact_to_dense(const uint32_t *head, const uint16_t *idx, const float *val, int slots, int N,
                           int nx, int ny, int nz, void *phi, int phi_dtype, void *stream);

/* Initial state from a grain-owner map and a z profile (the 3-D analogue of
 * init_phi_from_grain_map_3d, src/seed_modes_3d.py:38-57): owner int32
 * [slab][ny][nx] (x fastest) gives the grain of the first `slab` layers,
 * higher layers repeat layer slab-1; the grain holds prof[k] (float [nz]),
 * the liquid clip(1 - prof[k], 0, 1).  No dense phi is formed, so domains
 * whose dense field would not fit (e.g. 1024 x 1024 x 256 with 513 phases)
 * start directly in compact form. */
int mpf3d_compact_init_owner(const int32_t *owner, int slab, const float *prof, int nx, int ny, int nz,
                             int slots, uint32_t *head, uint16_t *idx, float *val, void *stream);

/* nf of the reference's APT (kernel_update_nfmf_3d, src/gpu_kernels_3d.py:462-486)
 * computed from a compact state, dense z-fastest int32 output. */
int mpf3d_compact_active_count(const uint32_t *head, const uint16_t *idx, int slots, int nx, int ny, int nz,
                               int32_t *nf, void *stream);

/* One time step in FP32 (three kernels): APT rebuild (src/gpu_kernels_3d.py:462-486),
 * phase update of kernel_update_phasefield_active_3d_switchable (:683-830)
 * and the cooling of kernel_update_temp_3d (:833-838) folded into
 * T = T0z[k] - (Tm_plus_cool - T_melt).  (slots, amax) is (4, 8), (8, 16) or
 * (16, 32); more active phases than amax, or more positive phases than
 * slots, leave the cell unchanged and set MPF3D_DEV_SLOT_OVERFLOW.
 * a2ij = aij*aij elementwise (float32).  T0z: float64 [nz].
 * symmetric_normals != 0 asserts that every grain's n111 rows 4..7 are the
 * exact negatives of rows 3..0 (true for the rotated (+-1,+-1,+-1)/sqrt(3)
 * set of src/orientation_utils.py:182-212), which halves the facet search
 * (the interface kernel is built once for 4 and once for 8 normals).
 * Scratch: work_items uint32[cells] (cells handed from the sweep kernel to
 * the general and interface kernels of the step) and work_count uint32[4],
 * zeroed once before the first step; `parity` alternates 0/1 on consecutive
 * steps so no reset is needed in between.  Cells must number fewer than 2^31.
 * Streams: with anisotropy on, the interface kernel runs on a library-owned
 * second stream, beside the general kernel, forked from and joined back to
 * `stream` by events; to the caller the step is ordered on `stream` like one
 * kernel.  Each caller stream of each device gets its own second stream and
 * event pair, created by its first such call made outside a stream capture;
 * a call inside a capture before that launches both kernels on `stream`.
 * Steps that callers issue on independent streams therefore stay
 * independent.  The same holds for mpf3d_compact_step_tuned,
 * mpf3d_compact_step_clocked and mpf3d_compact_step_noalloc; the batched step
 * (mpf3d_batched_step) runs on `stream` alone.  The second streams and events
 * live until the process ends; cudaDeviceReset is not supported after a
 * step. */
/* Creates the second stream of `stream` on the current device (see
 * "Streams" above) now, so that steps captured from `stream` into a CUDA
 * graph later run their general and interface kernels side by side.  Fails
 * (MPF3D_ERR_CUDA) when `stream` is being captured.  Optional: the first
 * uncaptured step on `stream` does the same. */
int mpf3d_streams_prepare(void *stream);

int mpf3d_compact_step(const uint32_t *head, const uint16_t *idx, const float *val, uint32_t *head_out,
                       uint16_t *idx_out, float *val_out, int slots, int amax, const double *T0z,
                       double Tm_plus_cool, const float *wij, const float *a2ij, const float *mij,
                       const float *n111, int N, int nx, int ny, int nz, const mpf3d_scalars *scalars,
                       int enable_anisotropy, int enable_torque, int symmetric_normals,
                       uint32_t *work_items, uint32_t *work_count, int parity, int32_t *err,
                       void *stream);

/* Launch shape of the compact step (see mpf3d_compact_step_tuned).  Every
 * shape computes the same result; only the scheduling differs. */
typedef struct mpf3d_tuning {
    int32_t sweep_zb;              /* cells per sweep thread along z: 2, 4 or 8 */
    int32_t sweep_by;              /* sweep block = 32 x sweep_by threads: 4, 8 or 16 */
    int32_t general_blocks_per_sm; /* general work-list kernel: blocks per SM, 1..64 */
    int32_t general_threads;       /* and threads per block: 128 or 256 */
    int32_t iface_blocks_per_sm;   /* interface work-list kernel: blocks per SM, 1..64 */
    int32_t iface_threads;         /* and threads per block: 64 or 128 */
} mpf3d_tuning;

/* mpf3d_compact_step with an explicit launch shape (NULL: the default
 * {4, 8, 8, 256, 8, 128}), as chosen by the package's autotuner, and
 * optional quiet-tile flags.  No reference counterpart: the reference
 * launches a fixed [4, 4, 4] block (config_3d.yaml gpu.threads_per_block)
 * over every cell.
 *
 * tile_flags (uint8, mpf3d_compact_tile_flags_len bytes, or NULL): per
 * 32 x 1 x sweep_zb tile of the sweep, "every cell was uniform" for the last
 * two steps (alternating halves by parity).  A tile that was uniform with
 * its 6 neighbours in the previous step is skipped -- no reads, no writes:
 * the output buffer already holds its cells.  The result is identical to
 * tile_flags = NULL.  Zero the whole array whenever the state buffers are
 * written other than by this function (initialisation, restore, rollback)
 * or sweep_zb changes; steps must alternate parity.  options: an OR of
 * MPF3D_STEP_MULTI_LIST and MPF3D_STEP_SWEEP_TMA. */
int mpf3d_compact_step_tuned(const uint32_t *head, const uint16_t *idx, const float *val, uint32_t *head_out,
                             uint16_t *idx_out, float *val_out, int slots, int amax, const double *T0z,
                             double Tm_plus_cool, const float *wij, const float *a2ij, const float *mij,
                             const float *n111, int N, int nx, int ny, int nz, const mpf3d_scalars *scalars,
                             int enable_anisotropy, int enable_torque, int symmetric_normals,
                             uint32_t *work_items, uint32_t *work_count, int parity, int32_t *err,
                             void *stream, const mpf3d_tuning *tuning, uint8_t *tile_flags, int options);

/* options of mpf3d_compact_step_tuned */
#define MPF3D_STEP_MULTI_LIST 1 /* interface cells whose neighbourhood holds two or more solids (decided
                                 * from the heads) get a work list of their own at
                                 * work_items[cells .. 2*cells): work_items must then hold 2*cells
                                 * entries and work_count 6.  Same results, fewer idle lanes. */

#define MPF3D_STEP_SWEEP_TMA 2 /* the sweep stages each block's heads plus a one-cell halo in shared memory
                                * with one TMA copy (cp.async.bulk.tensor.3d) and classifies from there;
                                * needs nx a multiple of 4 (otherwise the plain sweep runs).  Same
                                * results. */

/* Bytes of tile_flags for an nx x ny x nz domain (any sweep_zb). */
int64_t mpf3d_compact_tile_flags_len(int nx, int ny, int nz);

/* Device step clock of mpf3d_compact_step_clocked (device memory, 8-byte
 * aligned).  step[parity] holds the index of the step about to run with that
 * parity; the caller sets it once (step[n & 1] = n before step n) and each
 * step advances it.  tmc[] is written by the step for its own kernels. */
typedef struct mpf3d_step_clock {
    int64_t step[2];
    double tmc[2];
} mpf3d_step_clock;

/* mpf3d_compact_step_tuned with the step's temperature taken from the device:
 * the step reads its index s = clock->step[parity], runs at
 * Tm_plus_cool = T_melt + s * cooling_rate (float64, rounded operation by
 * operation: the same value as the host computing that expression) and
 * sets clock->step[parity ^ 1] = s + 1.  Nothing of the step is then passed
 * by value but its parity, so a CUDA graph of an even number of captured
 * steps can be replayed over and over and keeps cooling (the reference's
 * kernel_update_temp_3d, src/gpu_kernels_3d.py:833-838, applied once per
 * step).  Same results as mpf3d_compact_step_tuned at the same step index. */
int mpf3d_compact_step_clocked(const uint32_t *head, const uint16_t *idx, const float *val, uint32_t *head_out,
                               uint16_t *idx_out, float *val_out, int slots, int amax, const double *T0z,
                               mpf3d_step_clock *clock, double T_melt, double cooling_rate, const float *wij,
                               const float *a2ij, const float *mij, const float *n111, int N, int nx, int ny,
                               int nz, const mpf3d_scalars *scalars, int enable_anisotropy, int enable_torque,
                               int symmetric_normals, uint32_t *work_items, uint32_t *work_count, int parity,
                               int32_t *err, void *stream, const mpf3d_tuning *tuning, uint8_t *tile_flags,
                               int options);

/* compact state -> dense phi of one domain stored at cells [base, base +
 * nx*ny*nz) of state arrays whose slot planes are `stride` cells apart. */
int mpf3d_compact_to_dense_view(const uint32_t *head, const uint16_t *idx, const float *val, int slots,
                                uint32_t stride, uint32_t base, int N, int nx, int ny, int nz, void *phi,
                                int phi_dtype, void *stream);

/* ---- observables, slices and checkpoints of a compact state -------------- */

/* Reductions of compute_metrics_3d (tests/verification_3d.py:612-654) over
 * the dense field the compact state stands for (unstored phases are 0). */
typedef struct mpf3d_metrics {
    double solid_sum;      /* sum over cells of 1 - phi_liquid */
    double sum_err_max;    /* max over cells of |sum_g phi_g - 1| */
    double phi_min;        /* min over every (phase, cell) entry */
    double phi_max;        /* max over every (phase, cell) entry */
    double front_sum;      /* sum of the column front heights (cells) */
    double front_sq_sum;   /* sum of their squares */
    double front_max;      /* highest column front */
    int64_t nan_count;     /* NaN entries */
    int64_t front_columns; /* columns holding solid above the threshold */
    int32_t nf_max;        /* longest active-phase list (APT rule of kernel_update_nfmf_3d) */
    int32_t reserved;
} mpf3d_metrics;

/* Metrics of one compact state into the device struct `result`; optional
 * grain_sum (double[N], device) receives sum_cells phi_g for g >= 1 and
 * front (float[ny][nx], device) the highest z whose solid fraction exceeds
 * `threshold` per column, NaN where none (interface_positions_3d,
 * tests/verification_3d.py:409-416). */
int mpf3d_compact_metrics(const uint32_t *head, const uint16_t *idx, const float *val, int slots, int N,
                          int nx, int ny, int nz, float threshold, mpf3d_metrics *result, double *grain_sum,
                          float *front, void *stream);

/* One 2D slice (axis 0: xy at z = index, 1: xz at y = index, 2: yz at x =
 * index), row-major [W][H] with (W, H) = (nx, ny), (nx, nz) or (ny, nz):
 * ids = argmax phase (first maximum, as numpy.argmax over the phase axis of
 * save_phase_map_slice_3d, src/plot_utils_3d.py:36-72), vmax = its
 * fraction, solid = 1 - phi_liquid (save_solid_slice,
 * run_orientation_scan_3d.py:199-223).  Null outputs are skipped. */
int mpf3d_compact_slice(const uint32_t *head, const uint16_t *idx, const float *val, int slots, int nx, int ny,
                        int nz, int axis, int index, int32_t *ids, float *vmax, float *solid, void *stream);

/* Checkpoints (no reference counterpart: the reference keeps no restart
 * state).  A packed state is the head array plus the (id, value) entries of
 * every cell that keeps values, cell-major, ascending ids; implicit single
 * phases take no entry.  Offsets are recomputed from the heads, so head +
 * entries is the whole checkpoint.  scratch: int64[mpf3d_compact_pack_scratch_len(cells)]. */
int64_t mpf3d_compact_pack_scratch_len(int64_t cells);

/* Writes the entry count to *total (device int64).  With ids_out/vals_out
 * null only counts; otherwise writes entries that fit in `capacity`
 * (entries past it set MPF3D_DEV_BAD_INPUT in *err). */
int mpf3d_compact_pack(const uint32_t *head, const uint16_t *idx, const float *val, int slots, int64_t cells,
                       int64_t *scratch, int64_t *total, uint16_t *ids_out, float *vals_out, int64_t capacity,
                       int32_t *err, void *stream);

/* Inverse of mpf3d_compact_pack into a state whose head array already holds
 * the saved heads.  A cell with more entries than `slots` sets
 * MPF3D_DEV_SLOT_OVERFLOW, entries past n_entries or a first id that
 * disagrees with the head set MPF3D_DEV_BAD_INPUT. */
int mpf3d_compact_unpack(const uint32_t *head, const uint16_t *ids_in, const float *vals_in, int64_t n_entries,
                         int slots, int64_t cells, int64_t *scratch, uint16_t *idx_out, float *val_out, int32_t *err,
                         void *stream);

/* ---- batched instances (bicrystal / orientation-scan batches) -----------
 * No reference counterpart: the reference runs one domain at a time
 * (run_orientation_scan_3d.py:686-841, tests/verification_3d.py:1951-2011).
 * Instances share one compact state; instance i owns cells [offset,
 * offset + nx*ny*nz).  The table lives in DEVICE memory, sorted by offset
 * and tile_start, where tile_start is the first sweep tile of the instance
 * (tiles are 32 x 8 x 4 cells: ceil(nx/32)*ceil(ny/8)*ceil(nz/4) per
 * instance).  Temperature is uniform per instance (T_melt - undercooling),
 * anisotropy strength and grain orientations per instance. */
typedef struct mpf3d_instance {
    int32_t nx, ny, nz;
    uint32_t offset;      /* first cell of the instance */
    int32_t n111_base;    /* first n111 row of the instance's phases */
    int32_t split;        /* bicrystal: grain 1 for x < split, grain 2 for x >= split */
    int32_t tile_start;   /* first sweep tile of the instance */
    float delta_a;        /* anisotropy strength */
    float mu_da;          /* float(mu_a * delta_a) */
    float e2_flat;        /* float((eps0_sl * a(theta at cos 0))^2) for this delta_a */
    float undercooling;   /* T_melt - T */
    float base_height;    /* bicrystal: initial solid height in cells */
} mpf3d_instance;

/* Bicrystal initial state of every instance: a tanh solid base of
 * base_height cells (src/seed_modes_3d.py:46-56 profile), grain 1 left of
 * `split`, grain 2 right of it, liquid above. */
int mpf3d_batched_init_bicrystal(const mpf3d_instance *inst, int n_inst, uint32_t total_cells, double dx,
                                 double delta, uint32_t *head, uint16_t *idx, float *val, int32_t *err,
                                 void *stream);

/* One step of every instance: the three step kernels of mpf3d_compact_step
 * launched once over the whole batch.  n_tiles = total sweep tiles.  Shared
 * physics from `scalars` (delta_a there is ignored); the rest as
 * mpf3d_compact_step_tuned with total_cells in place of nx*ny*nz (options:
 * 0 or MPF3D_STEP_MULTI_LIST). */
int mpf3d_batched_step(const uint32_t *head, const uint16_t *idx, const float *val, uint32_t *head_out,
                       uint16_t *idx_out, float *val_out, int slots, int amax, const mpf3d_instance *inst,
                       int n_inst, int n_tiles, uint32_t total_cells, const float *wij, const float *a2ij,
                       const float *mij, const float *n111, int N, const mpf3d_scalars *scalars,
                       int enable_anisotropy, int enable_torque, int symmetric_normals, uint32_t *work_items,
                       uint32_t *work_count, int parity, int32_t *err, void *stream, int options);

/* mpf3d_batched_step with the grids and block sizes of the two work-list
 * kernels from `tuning` (its general_* and iface_* fields; the sweep's 32 x 8 x
 * 4 tiles are fixed by the instance table, so sweep_zb and sweep_by must be
 * valid but are not used).  NULL: {8 x 256, 8 x 128} blocks per SM.  Every
 * shape computes the same result.
 *
 * tile_flags (uint8, mpf3d_batched_tile_flags_len(n_tiles) bytes, or NULL):
 * quiet-tile flags of the batched sweep, as for mpf3d_compact_step_tuned,
 * per 32 x 1 x 4 warp tile of each instance.  Zero them before the first
 * step and whenever the state buffers are written other than by this
 * function (initialisation, restore); steps must alternate parity.  Same
 * results with and without them. */
int mpf3d_batched_step_tuned(const uint32_t *head, const uint16_t *idx, const float *val, uint32_t *head_out,
                             uint16_t *idx_out, float *val_out, int slots, int amax, const mpf3d_instance *inst,
                             int n_inst, int n_tiles, uint32_t total_cells, const float *wij, const float *a2ij,
                             const float *mij, const float *n111, int N, const mpf3d_scalars *scalars,
                             int enable_anisotropy, int enable_torque, int symmetric_normals, uint32_t *work_items,
                             uint32_t *work_count, int parity, int32_t *err, void *stream, int options,
                             const mpf3d_tuning *tuning, uint8_t *tile_flags);

/* bytes of the batched step's quiet-tile flags: 2 parities x 8 warp tiles
 * per sweep tile (0 for n_tiles <= 0) */
int64_t mpf3d_batched_tile_flags_len(int n_tiles);

/* Observables per instance, accumulated into zeroed float64 arrays:
 * acc[6*i..6*i+5] = {sum of front heights left of split, columns left, sum
 * right, columns right, sum phi1, sum phi2}; the front of a column is the
 * highest z whose solid fraction exceeds 0.5 (interface_positions_3d,
 * tests/verification_3d.py:409-416). */
int mpf3d_batched_fronts(const uint32_t *head, const uint16_t *idx, const float *val, int slots,
                         const mpf3d_instance *inst, int n_inst, uint32_t total_cells, double *acc,
                         void *stream);

/* Grain-boundary rows: for every z row of every instance with solid
 * fraction >= 0.15, the phi1 = phi2 crossing along x nearest `split`
 * (measure_gb_inclination, tests/run_paper_verification.py:658-723) summed
 * over y: gb[2*(row_base[i] + k)] += x, gb[2*(row_base[i] + k) + 1] += 1.
 * row_base (device, int32[n_inst]) = running sum of nz. */
int mpf3d_batched_gb_rows(const uint32_t *head, const uint16_t *idx, const float *val, int slots,
                          const mpf3d_instance *inst, int n_inst, uint32_t total_cells, const int32_t *row_base,
                          double *gb, void *stream);

/* Orientation-scan set-up: instance i holds a sphere of phase `solid_gid`
 * of radius[i] cells centred at center[3i..3i+2] (cell units, index * dx is
 * the position), liquid elsewhere, with the tanh profile of
 * init_singlemode_sphere_3d (src/seed_modes_3d.py:59-113). */
int mpf3d_batched_init_sphere(const mpf3d_instance *inst, int n_inst, uint32_t total_cells, double dx,
                              double delta, const float *center, const float *radius, int solid_gid, int slots,
                              uint32_t *head, uint16_t *idx, float *val, void *stream);

/* Directional radii of measure_observables (run_orientation_scan_3d.py:
 * 292-351): per instance i, direction d and sign (+, -), the distance in
 * cells from center[3i..] along +-dirs[3d..] at which the trilinear
 * interpolant of `phase` drops below `threshold`, marching in steps of
 * step_cells; NaN where it does not.  out[(i*n_dir + d)*2 + sign]. */
int mpf3d_batched_ray_radii(const uint32_t *head, const uint16_t *idx, const float *val, int slots,
                            const mpf3d_instance *inst, int n_inst, uint32_t total_cells, int phase,
                            const float *center, const float *dirs, int n_dir, double threshold, double step_cells,
                            double *out, void *stream);

/* ---- surrogate network kernels (BF16 tensor cores, FP32 accumulate) ------
 * No reference counterpart: the reference has no learned component.  BF16
 * values are passed as uint16_t bit patterns. */

/* C[m][n] = act(sum_k A(m,k) B(k,n) + bias[n]) with A(m,k) = A[m*sam + k*sak],
 * B(k,n) = B[k*sbk + n*sbn]; act 0 = none, 1 = SiLU.  Z (nullable) receives
 * the FP32 pre-activation, Y the result (BF16 if y_bf16, else FP32, added to
 * Y when beta = 1), both with row stride ldy.  K-major operands that fit
 * mpf3d_gemm_bf16_tc5 run there, other layouts on
 * mpf3d_gemm_bf16_tc5_strided, shapes neither covers on
 * mpf3d_gemm_bf16_mma.  err
 * (nullable device word) receives MPF3D_DEV_GEMM_ABORT from the tcgen05
 * kernel. */
int mpf3d_gemm_bf16(int M, int N, int K, const uint16_t *A, int64_t sam, int64_t sak, const uint16_t *B,
                    int64_t sbk, int64_t sbn, const float *bias, int act, float *Z, void *Y, int ldy,
                    int y_bf16, int beta, int32_t *err, void *stream);

/* The two kernels behind mpf3d_gemm_bf16, callable directly.  _tc5: the
 * tcgen05 kernel (M x N tiles of 128 x N in tensor memory) for K-major A
 * [M][K] (row stride lda) and B given as [N][K] (row stride ldb), K a
 * multiple of 16 up to 256, N up to 256, 16-byte aligned rows; other shapes
 * return MPF3D_ERR_ARG.  _mma: the mma.sync kernel, any strides.
 * Every mbarrier wait of the tcgen05 kernel is bounded (1 s).  A wait that
 * runs out stops the CTA's work: the MMAs already issued and the copies in
 * flight are waited for (again bounded) before the tensor memory is freed,
 * the CTA's output rows are written as NaN and MPF3D_DEV_GEMM_ABORT is OR-ed
 * into *err (nullable). */
int mpf3d_gemm_bf16_tc5(int M, int N, int K, const uint16_t *A, int64_t lda, const uint16_t *B, int64_t ldb,
                        const float *bias, int act, float *Z, void *Y, int ldy, int y_bf16, int beta, int32_t *err,
                        void *stream);

/* The tcgen05 kernel for operands in any layout -- A(m,k) = A[m*sam + k*sak],
 * B(k,n) = B[k*sbk + n*sbn] as in mpf3d_gemm_bf16 -- which gathers them into
 * the K-major shared-memory layout (the gradients dZ W and dZ^T X of the
 * surrogate read transposed operands).  N <= 256, any K: the reduction is
 * staged in blocks of up to 256 (zero-padded to a multiple of 16), and a
 * reduction deeper than 256 is accumulated block by block into an FP32 Y
 * (then act must be 0, Z null and y_bf16 0). */
int mpf3d_gemm_bf16_tc5_strided(int M, int N, int K, const uint16_t *A, int64_t sam, int64_t sak, const uint16_t *B,
                                int64_t sbk, int64_t sbn, const float *bias, int act, float *Z, void *Y, int ldy,
                                int y_bf16, int beta, int32_t *err, void *stream);

/* The pipelined tcgen05 kernel of mpf3d_gemm_bf16_tc5 (K a multiple of 64)
 * with its TMA producer held back, so that no copy and no MMA is ever issued
 * and every wait of the other roles runs out after wait_ns (at most 0.1 s):
 * a test of the abort path.  Expected result: MPF3D_DEV_GEMM_ABORT in *err
 * (required) and NaN in Y.  No reference counterpart. */
int mpf3d_gemm_bf16_tc5_held(int M, int N, int K, const uint16_t *A, int64_t lda, const uint16_t *B, int64_t ldb,
                             void *Y, int ldy, int32_t *err, uint64_t wait_ns, void *stream);
int mpf3d_gemm_bf16_mma(int M, int N, int K, const uint16_t *A, int64_t sam, int64_t sak, const uint16_t *B,
                        int64_t sbk, int64_t sbn, const float *bias, int act, float *Z, void *Y, int ldy,
                        int y_bf16, int beta, void *stream);

/* dZ = dY * act'(Z) elementwise; outputs BF16 and/or FP32 (each nullable). */
int mpf3d_act_backward(const float *dY, const float *Z, int act, int64_t n, uint16_t *dZ16, float *dZ32,
                       void *stream);

/* out[n] = sum over m of X[m*ld + n]. */
int mpf3d_colsum(const float *X, int M, int N, int ld, float *out, void *stream);

/* Weighted MSE of the first n_out columns of pred (row stride ld) against
 * target [M][n_out]: *loss += sum w_c (pred - t)^2 / M, dpred = its gradient. */
int mpf3d_mse(const float *pred, int ld, const float *target, int M, int n_out, const float *w, float *dpred,
              float *loss, void *stream);

/* Adam step `step` (1-based) on FP32 weights with decoupled weight decay
 * folded into the gradient; w16 (nullable) receives the BF16 copy. */
int mpf3d_adam(float *w, float *m, float *v, const float *g, uint16_t *w16, int64_t n, float lr, float b1,
               float b2, float eps, int step, float weight_decay, void *stream);

/* FP32 -> BF16, round to nearest even. */
int mpf3d_f32_to_bf16(const float *x, uint16_t *y, int64_t n, void *stream);

/* Largest grid (nx*ny*nz) that mpf3d_compact_step_noalloc accepts. */
#define MPF3D_NOALLOC_MAX_CELLS 4194304u

/* mpf3d_compact_step without caller scratch and without any device
 * allocation.  No counterpart in the reference: it serves hosts that cannot
 * let a library allocate device memory -- applications that reserve the whole
 * memory budget up front for their own pool, or real-time loops where a
 * cudaMalloc (which may synchronise the device) is not acceptable.
 * The step's work list lives in a file-scope device array of
 * MPF3D_NOALLOC_MAX_CELLS entries (16 MiB, plus 16 bytes of counters) that
 * every GPU loading the library holds until the process exits; larger grids
 * return MPF3D_ERR_TOO_LARGE.  The first call on a device looks up the
 * array's device address with that device current; make that first call
 * before any stream capture.  All calls share the array and the call clears
 * its counters on `stream` first, so calls that overlap on the GPU (other
 * streams, other host threads) race on it: serialise them.  The device
 * address is looked up once per device and kept: a cudaDeviceReset after a
 * call on that device is not supported.  Other arguments and results are
 * those of mpf3d_compact_step (parity is not needed). */
int mpf3d_compact_step_noalloc(const uint32_t *head, const uint16_t *idx, const float *val,
                               uint32_t *head_out, uint16_t *idx_out, float *val_out, int slots, int amax,
                               const double *T0z, double Tm_plus_cool, const float *wij, const float *a2ij,
                               const float *mij, const float *n111, int N, int nx, int ny, int nz,
                               const mpf3d_scalars *scalars, int enable_anisotropy, int enable_torque,
                               int symmetric_normals, int32_t *err, void *stream);

/* library version, for the binding's load check */
int mpf3d_version(void);

#ifdef __cplusplus
}
#endif
#endif /* MPF3D_H */
