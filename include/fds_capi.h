/*
 * fds_capi.h -- C ABI of libfdsgpu.so, the GB300 engine behind pyfds_gb300.
 *
 * The reference (emtpb/pyfds) is pure Python: its hot path is
 * `Field.simulate()` (pyfds/fields.py:67-95) calling each field's `sim_step()`
 * (pyfds/acoustics.py:40-52, 111-128, 205-225; pyfds/thermal.py:40-51, 92-107,
 * 161-176), which applies scipy.sparse DIA operators built by
 * `assemble_matrices()` and applies boundaries / records outputs
 * (pyfds/fields.py:591-611, pyfds/regions.py:125-165). This ABI replaces that
 * loop: one call advances a field by `nsteps` steps on the GPU, with the same
 * boundary and output semantics, over device buffers the caller owns.
 *
 * Conventions
 *  - Every pointer in these structs is a DEVICE pointer unless stated; the caller
 *    allocates and owns all memory (PyTorch tensors in pyfds_gb300). The library
 *    borrows pointers for the duration of a call and retains none.
 *  - Work is enqueued on `stream` (a cudaStream_t passed as void*; NULL = legacy
 *    default stream). Calls return after enqueueing; they do not synchronise.
 *  - Return value: 0 on success, a negative FDS_E* code on failure; the message
 *    of the last failure on the calling thread is available from fds_last_error.
 *  - Calls may come from several host threads and for several devices of one
 *    process, each on its own problem, state and stream (the device is the
 *    calling thread's current one); fds_stag_batch_run_static is the exception
 *    (one shared workspace, see there).
 *  - Flat cell index i = x + y * nx (pyfds/fields.py:377); a 1-D field has ny = 1.
 *    Neighbours are i +- 1 and i +- nx with NO break at row ends: only indices
 *    outside [0, nx*ny) are dropped, as in the reference's truncated DIA operators.
 */
#ifndef FDS_CAPI_H
#define FDS_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 3: FdsBoundGroup.primary (was padding; kernels that apply bounds to global arrays
 *    read it), FdsStagProblem.stages = 3, FDS_PREC_DW, fds_dw_split / fds_dw_join */
#define FDS_ABI_VERSION 5

/* error codes */
#define FDS_OK 0
#define FDS_E_ARG (-1)       /* invalid argument (null pointer, bad size, unknown mode) */
#define FDS_E_LAUNCH (-2)    /* a CUDA launch or API call failed */
#define FDS_E_NOKERNEL (-3)  /* no kernel was built for this combination of flags */
#define FDS_E_TIMEOUT (-4)   /* a bounded device-side wait gave up */
#define FDS_E_SIZE (-5)      /* a size exceeds a documented maximum */

/* field families (FdsStagProblem.family) */
#define FDS_FAMILY_ACOUSTIC 0 /* flux components keep memory: v -= (D p - L v) */
#define FDS_FAMILY_THERMAL 1  /* flux components are overwritten: q = -(D T) */

/* arithmetic (FdsStagProblem.precision) */
#define FDS_PREC_F64 0     /* all state and coefficients float64 (the drop-in) */
#define FDS_PREC_F32 1     /* all state and coefficients float32 */
#define FDS_PREC_F32_T64 2 /* float32 coefficients and fluxes, float64 potential (P/T) */
#define FDS_PREC_DW 3      /* double-word: every state and coefficient value is a pair of
                              float32 {hi, lo} (8 bytes, value hi + lo, |lo| <= ulp(hi)/2)
                              computed with compensated float32 arithmetic (48-bit
                              significands); no register-marching tiles, not exact */

/* FdsStagProblem.flags */
#define FDS_FLAG_HAS_V 1u   /* second flux component (2-D fields) */
#define FDS_FLAG_ABSORB 2u  /* viscous absorption operator present (acoustic) */
#define FDS_FLAG_AXI 4u     /* axisymmetric: x is the radius (Acoustic3DAxi / Thermal3DAxi) */
#define FDS_FLAG_EXACT 8u   /* F64 only: reproduce the reference's floating-point
                              operation order exactly (no fused multiply-add) */
#define FDS_FLAG_FLOW 16u   /* acoustic 2-D with a moving medium (AcousticFlow2D): after
                              each step, rows y with flow_period[y] == 0 or
                              step % flow_period[y] == 0 move one cell in +x (their
                              first cell becomes 0) in p, vx and vy */

/* Boundary operation flags (FdsBoundOp.flags) */
#define FDS_BOP_SIGNAL 2 /* value = pool[off + step * stride]  (else value = scalar) */

/*
 * Per-cell coefficient arrays of one field. Each array has nx*ny entries of the
 * problem's coefficient type (double for F64, float otherwise) and is indexed by
 * the cell it multiplies, i.e. by column of the reference's DIA operator
 * (scipy stores data[k][j] at A[j - offset_k, j]).
 *
 *  bx, by : factors of the backward x / y difference that updates the flux
 *           (reference a_vx_p / a_vy_p: dt/dx/rho; thermal a_qx_t / a_qy_t: kx/dx).
 *  kx, ky : factors of the forward x / y difference that updates the potential
 *           (reference a_p_vx / a_p_vy: dt/dx*c^2*rho; thermal a_t_qx / a_t_qy:
 *           dt/dx/rho/cp). For FDS_FLAG_AXI with FDS_FLAG_EXACT these carry the
 *           reference's 1/r column factor and the kernel multiplies the flux by r.
 *  absorption (FDS_FLAG_ABSORB, else NULL): the summed DIA operator
 *           a_vx_vx = (d_x2 + d_y2 [+ central d_x for AXI]).todia(), as its
 *           diagonals: aym (offset -nx), axm (offset -1), ad (offset 0),
 *           axp (offset +1), ayp (offset +nx); each column-indexed.
 *  ex     : AXI + ABSORB only: dt*mu/rho, the explicit radial loss of
 *           pyfds/acoustics.py:213-215.
 *  rx     : AXI only: radius of each column, nx entries (x_j + dx/2).
 */
typedef struct FdsCoefs {
  const void* bx;
  const void* by;
  const void* kx;
  const void* ky;
  const void* aym;
  const void* axm;
  const void* ad;
  const void* axp;
  const void* ayp;
  const void* ex;
  const void* rx;
} FdsCoefs;

/* Geometry and variant of one staggered field. */
typedef struct FdsStagProblem {
  int32_t family;    /* FDS_FAMILY_* */
  int32_t precision; /* FDS_PREC_* */
  uint32_t flags;    /* FDS_FLAG_* */
  int32_t nx;
  int32_t ny; /* 1 for 1-D fields */
  int32_t tile_x; /* tile shape the tables below were built for: the default of */
  int32_t tile_y; /* fds_stag_tile_shape, or for lossless 2-D non-exact variants any
                     shape listed by fds_stag_tile_menu */
  int32_t stages; /* 0 (automatic) or 1: one CTA per tile; 2: persistent CTAs that
                     prefetch the next tile while computing one (lossless 2-D variants);
                     3: two steps per tile and launch (lossless 2-D, non-exact, no
                     moving medium, not float32-with-float64-potential; tables in slot
                     layout 2, see fds_stag_tile_menu);
                     4: every step of the call in one persistent launch (lossless 2-D,
                     non-exact, no moving medium, default tile shape; slot layout 0):
                     CTAs take (step, tile) items in order from a queue and wait,
                     bounded, until the tile rows around their tile finished the
                     previous step; needs FdsStagTables.sync */
  FdsCoefs coefs;
  double offset;  /* thermal float32 only: the temperature is stored as T - offset
                     (finer float spacing near a reference temperature); the flux
                     adds the reference's interface term -(b_i - b_i-1) * offset, and
                     boundary values / outputs are shifted by the caller. 0 otherwise */
  const int64_t* flow_period; /* FDS_FLAG_FLOW: [ny] device array of shift periods in
                                 steps, int(dx / flow / dt) per row; NULL otherwise */
  const int64_t* flow_period_host; /* FDS_FLAG_FLOW, optional: the same periods in host
                                      memory; steps on which no row is due then skip
                                      the shift launch and step as a field at rest */
} FdsStagProblem;

/*
 * Field state, ping-pong buffered. Component 0 is the potential (pressure /
 * temperature), 1 and 2 the x / y flux (velocity / heat flux). `cur[c]` holds the
 * current values; `nxt[c]` is scratch of the same size. On return the pointers
 * are swapped as many times as steps ran, so `cur[c]` again holds the current
 * values. A thermal flux component may pass cur == nxt (it is never read).
 */
typedef struct FdsStagState {
  void* cur[3];
  void* nxt[3];
} FdsStagState;

/* One boundary operation (pyfds/regions.py:125-145):
 *   new = mul * old + value,
 * where mul is the boundary's `additive` flag as a number (True -> 1, False -> 0,
 * as the reference multiplies it in). 32 bytes. */
typedef struct FdsBoundOp {
  double scalar;  /* value when !(flags & FDS_BOP_SIGNAL); with FDS_BOP_SIGNAL a
                     constant added to the signal sample (0 unless the potential is
                     stored with an offset) */
  double mul;     /* factor of the old value */
  int64_t off;    /* pool offset of step 0 when FDS_BOP_SIGNAL */
  int32_t stride; /* pool stride between consecutive steps */
  int32_t flags;  /* FDS_BOP_* */
} FdsBoundOp;

/* One boundary cell of one tile: the chain ops[op_begin, op_end) applied in order
 * to the tile's shared-memory slot `pos`; `cell` is the flat index. A cell can sit
 * in several tiles' slots (halos that a tile recomputes); `primary` is 1 for one of
 * them (the owning tile's), and the first-step prologue, which works on the global
 * array, applies only primary groups. 24 bytes. */
typedef struct FdsBoundGroup {
  int64_t cell;
  int32_t pos;
  int32_t op_begin;
  int32_t op_end;
  int32_t primary;
} FdsBoundGroup;

/* One output sample slot: column `col` of the component's output buffer reads
 * the tile slot `pos` (flat index `cell`). 16 bytes. */
typedef struct FdsProbe {
  int64_t cell;
  int32_t pos;
  int32_t col;
} FdsProbe;

/* Boundary + output tables of one component, bucketed per tile. */
typedef struct FdsCompTables {
  const int32_t* bound_tile_start; /* [ntiles + 1] into groups, or NULL if none */
  const FdsBoundGroup* groups;
  const FdsBoundOp* ops;
  const int32_t* probe_tile_start; /* [ntiles + 1] into probes, or NULL if none */
  const FdsProbe* probes;
  double* out;  /* [nsteps_capacity, ncols] float64, row = step - step0 */
  int32_t ncols;
  int32_t out_rows; /* capacity of `out` in rows */
} FdsCompTables;

typedef struct FdsStagTables {
  FdsCompTables comp[3];
  const double* pool; /* boundary signal values, float64 */
  int64_t pool_len;
  int32_t* status;    /* device int32 the kernels OR FDS_STATUS_* bits into, or NULL;
                         the caller zeroes it and reads it after the stream work */
  uint32_t* sync;     /* stages 4 only: device scratch of fds_stag_sync_words() words
                         (the library zeroes them before each launch); NULL otherwise */
  int64_t sync_words; /* capacity of `sync` in 32-bit words */
} FdsStagTables;

/* Bits of FdsStagTables.status */
#define FDS_STATUS_TMA_TIMEOUT 1 /* a bounded wait gave up (TMA copies that did not
                                    land, or, with stages 4, tile rows of the previous
                                    step that did not finish); that tile was not
                                    updated and the state is not valid */
#define FDS_STATUS_NONFINITE 2   /* the potential of the call's last step holds a
                                    NaN or an infinity (the field diverged) */

/* ABI version of the loaded library (FDS_ABI_VERSION). */
int32_t fds_abi_version(void);

/* Copies the last error message of the calling thread into buf (NUL-terminated,
 * truncated to len). Returns the message length. */
int32_t fds_last_error(char* buf, size_t len);

/* Tile shape (cells in x, y) the kernel for this problem variant uses by default;
 * host-side tables must be bucketed for it: 1024 x 1 (1-D), 64 x 16 (2-D), 64 x 12
 * (2-D lossless double words). Returns FDS_OK or FDS_E_NOKERNEL. */
int32_t fds_stag_tile_shape(int32_t family, int32_t precision, uint32_t flags, int32_t nx,
                            int32_t ny, int32_t* tile_x, int32_t* tile_y);

/* Tile shapes built for the lossless 2-D variants (the autotuner's search space).
 * Writes up to `capacity` entries; returns how many exist. `layout` tells how the
 * host numbers the slots of a tile in FdsBoundGroup.pos / FdsProbe.pos:
 *   0 (shared-memory tile): pos = (ly + 1) * (tile_x + 8) + lx + 4   (1-D: ly + 0)
 *   1 (register marching):  pos = ly * (tile_x + 2) + lx + 1
 * with (lx, ly) the cell relative to the tile's first owned cell. (New: no
 * reference counterpart; tiling is a property of the GPU kernel.)
 * Two steps per tile (FdsStagProblem.stages = 3; tiles 64x16, 64x12, 64x8, 32x32)
 * use layout 2: pos = (ly + 2) * (tile_x + 8) + lx + 4, and a tile's bound groups
 * cover every slot of the ring it computes in its first step (potential: lx in
 * -1 .. tile_x, ly in -1 .. tile_y; x flux: lx up to tile_x + 1; y flux: ly up to
 * tile_y + 1), each cell once per flat-index alias, one placement flagged primary. */
int32_t fds_stag_tile_menu(int32_t* tile_x, int32_t* tile_y, int32_t* layout, int32_t capacity);

/*
 * Advance one staggered field by `nsteps` steps, steps step0 .. step0+nsteps-1.
 * Replaces `Field.simulate(nsteps)` (pyfds/fields.py:67-95) of Acoustic1D,
 * Acoustic2D, Acoustic3DAxi, Thermal1D, Thermal2D and Thermal3DAxi; each step
 * follows that kind's `sim_step()`:
 *   potential bounds(step) -> potential outputs -> flux update ->
 *   x-flux bounds -> x-flux outputs -> y-flux bounds -> y-flux outputs ->
 *   potential update.
 * `store_flux` != 0 writes the flux components every step (required for the
 * acoustic family, whose fluxes carry state); for the thermal family 0 writes
 * them on the last step only.
 */
int32_t fds_stag_run(const FdsStagProblem* prob, FdsStagState* state,
                     const FdsStagTables* tables, int64_t step0, int32_t nsteps,
                     int32_t store_flux, void* stream);

/* 32-bit words of FdsStagTables.sync that a stages-4 run of `prob` needs (one
 * work counter and one completion counter per row of tiles), or a negative error
 * code. The replaced reference loop is the same as fds_stag_run's. */
int64_t fds_stag_sync_words(const FdsStagProblem* prob);

/* ---------------------------------------------------------------- nonlinear 1-D
 * IdealGas1D and Acoustic2ndOrder1D (pyfds/nonlinear_acoustics.py:10-171): pressure,
 * velocity and density on a 1-D grid. One step: pressure bounds/outputs;
 *   v -= a_v_p p / (rho0 + d) [+ a_v_v2 v] - a_v_v v / (rho0 + d);
 * velocity bounds/outputs; d -= a_d_v ((d + rho0) v); density bounds/outputs; then
 * the state equation: ideal gas p = e1 ((rho0 + d) / rho0)^e2 - e1 (nonlinear,
 * e1 = rho0 c^2 / gamma, e2 = gamma, evaluated as e1 * (x^e2 - 1)) or p = e1 d
 * (linear, e1 = c^2); second order p = e1 d + e2 d^2 (e1 = d_rho_p, e2 = d_rho2_p / 2). */
#define FDS_NL1D_IDEAL_GAS 0
#define FDS_NL1D_SECOND_ORDER 1
#define FDS_NL1D_CONVECTIVE 1u /* the central a_v_v2 term (always on for second order) */
#define FDS_NL1D_NL_STATE 2u   /* ideal gas: nonlinear state equation */

typedef struct FdsNl1dProblem {
  int32_t kind;      /* FDS_NL1D_* */
  uint32_t flags;    /* FDS_NL1D_CONVECTIVE | FDS_NL1D_NL_STATE | FDS_FLAG_EXACT */
  int32_t n;         /* cells */
  int32_t tile_x;    /* tiling the boundary/output tables were bucketed for */
  double f1;         /* dt/dx: the diagonals of a_v_p (backward) and a_d_v (forward) */
  double fc;         /* (dt/dx/2)/2: the diagonals of the central a_v_v2 */
  const double* a;   /* [n] dt/dx^2 mu: the a_v_v diagonals (a, -2a, a) */
  const double* rho0;/* [n] static density */
  const double* e1;  /* [n] state-equation factor (see above) */
  const double* e2;  /* [n] state-equation factor or exponent (see above) */
  uint32_t* sync;    /* device uint32: the grid barrier's arrival counter (scratch; zeroed
                        by the call; calls sharing it must be stream-ordered) */
  int32_t* status;   /* device int32 the kernel ORs FDS_STATUS_* bits into, or NULL */
} FdsNl1dProblem;

/* Advances a nonlinear 1-D field by nsteps steps in one cooperative launch: one CTA
 * per tile of tile_x cells loops over the steps, with two grid-wide barriers per step
 * (bounded waits; FDS_STATUS_TMA_TIMEOUT is reported if one gives up). state->cur/nxt: pressure (updated in place in cur),
 * velocity and density (ping-pong, swapped per step like fds_stag_run). tables->comp:
 * pressure, velocity, density. Replaces the loop of Field.simulate around
 * IdealGas1D.sim_step / Acoustic2ndOrder1D.sim_step (pyfds/nonlinear_acoustics.py:55-90,
 * 140-163). */
int32_t fds_nl1d_run(const FdsNl1dProblem* prob, FdsStagState* state,
                     const FdsStagTables* tables, int64_t step0, int32_t nsteps, void* stream);

/* ThermoAcoustic1D (pyfds/coupled_fields.py:10-65) for nsteps steps in one call: per
 * step the acoustic step, the thermal step (both as fds_stag_run for one step; output
 * row = step - step0) and the loss coupling of BoundaryCoupling.apply
 * (pyfds/coupling.py:121-140) from the acoustic velocity into the temperature:
 *   loss = g * (a_v_p (v * rho_ac))^2 * dt, with a_v_p the acoustic backward
 *   difference of factor bx = dt/dx/rho_ac and g = (mu / rho_th) / c_th;
 *   stepping == 1 and !accumulate: T += loss every step; accumulate: acc += loss every
 *   step and, when step % stepping == 0, T += acc and acc is emptied; otherwise
 *   T += loss when step % stepping == 0.
 * acc: [n] device accumulator; *acc_empty (host, in/out) says it holds nothing yet.
 * Both problems must be float64 1-D fields of the same size. Fields of up to 2048
 * cells (with both in exact mode or both not) run every step of the call in one
 * launch on a thread-block cluster; the results are the per-step launches' bit for
 * bit. */
int32_t fds_thermoacoustic_run(const FdsStagProblem* acoustic, FdsStagState* ac_state,
                               const FdsStagTables* ac_tables, const FdsStagProblem* thermal,
                               FdsStagState* th_state, const FdsStagTables* th_tables,
                               const double* g, const double* rho_ac, double* acc,
                               int32_t* acc_empty, double dt, int32_t stepping,
                               int32_t accumulate, int64_t step0, int32_t nsteps, void* stream);

/* The moving-medium shift of one step alone, in place on state->cur (p, vx, vy):
 * replaces AcousticFlow2D.apply_flow (pyfds/acoustic_flow.py:49-57) for callers that
 * step a flow field themselves. Needs FDS_FLAG_FLOW and flow_period. */
int32_t fds_stag_flow_shift(const FdsStagProblem* prob, FdsStagState* state, int64_t step,
                            void* stream);

/* Double words (FDS_PREC_DW) on the device: fds_dw_split turns n float64 values
 * into {float hi, float lo} pairs (hi = (float)x, lo = (float)(x - hi), both rounded
 * to nearest), fds_dw_join adds pairs back into float64 ((double)hi + (double)lo).
 * Device pointers; `out` may not overlap `in`. (New: the host-side conversion of
 * pyfds_gb300, done where the data already is.) */
int32_t fds_dw_split(const double* in, void* out, int64_t n, void* stream);
int32_t fds_dw_join(const void* in, double* out, int64_t n, void* stream);

/* One array of a host gather: n float64 values at the HOST address src, written to
 * the DEVICE address dst as float64 (FDS_GATHER_F64), float32 rounded to nearest
 * (FDS_GATHER_F32) or double words as fds_dw_split forms them (FDS_GATHER_DW). */
typedef struct FdsGatherItem {
  const double* src;
  void* dst;
  int64_t n;
  int32_t kind;
  int32_t pad;
} FdsGatherItem;

#define FDS_GATHER_F64 0
#define FDS_GATHER_F32 1
#define FDS_GATHER_DW 2

/* 1 when the current device reads pageable host memory coherently through the
 * host's page tables (Grace-class hosts: NVLink-C2C with address translation), the
 * condition for fds_host_gather; 0 otherwise. */
int32_t fds_host_access(void);

/* Copies `count` host arrays to the device in one kernel that reads the caller's
 * pageable memory directly, converting each value as its item says; `items` is a
 * HOST array of `count` items. The arrays (and `items`) must stay valid until the
 * stream's work has finished. FDS_E_ARG where fds_host_access() is 0 or an item is
 * malformed. (New: replaces per-array host-to-device copies, each of which waits
 * for the stream, when a batch uploads the state and coefficients of many fields.) */
int32_t fds_host_gather(const FdsGatherItem* items, int32_t count, void* stream);

/* Workspace (device bytes, 256-byte aligned) a batched call over `count` instances
 * with `total_tiles` tiles in all needs: per-instance descriptors and the work
 * list. (New: no reference counterpart; the reference runs one field at a time.) */
size_t fds_stag_batch_workspace_bytes(int32_t count, int64_t total_tiles);

/*
 * Advance `count` independent fields by `nsteps` steps each with one kernel
 * launch per step covering every tile of every instance (plus one prologue
 * launch). Each instance i is `probs[i]` / `states[i]` / `tables[i]` exactly as
 * for fds_stag_run; all instances share family, precision, flags, tile and stages
 * (lossless 2-D, non-exact variants), and may differ in grid size and media.
 * Equivalent to calling fds_stag_run on each instance (the reference's
 * `Field.simulate`, pyfds/fields.py:67-95, once per field); the descriptors and
 * work list are written into the caller's `workspace` (see
 * fds_stag_batch_workspace_bytes) by an asynchronous copy on `stream`.
 * `mode`: FDS_BATCH_UPLOAD writes the descriptors (host work + a copy);
 * FDS_BATCH_LAUNCH enqueues the kernels only (no host-side copies, so it can be
 * captured into a CUDA graph) and needs a workspace uploaded with the same
 * arguments; both bits do both. After the launch phase the state pointers of
 * every instance are swapped as many times as steps ran.
 */
#define FDS_BATCH_UPLOAD 1u
#define FDS_BATCH_LAUNCH 2u
int32_t fds_stag_batch_run(const FdsStagProblem* probs, FdsStagState* states,
                           const FdsStagTables* tables, int32_t count, void* workspace,
                           size_t workspace_bytes, int64_t step0, int32_t nsteps,
                           int32_t store_flux, uint32_t mode, void* stream);

/*
 * Diagnostics: runs the kernels' bounded-wait helpers on waits that nothing
 * completes, with `poll_limit` polls (1 .. 2^20): mode 0 an mbarrier that no copy or
 * arrival targets (the TMA staging wait), mode 1 the device word `counter` (zero,
 * never incremented; the wavefront kernel's tile-row wait). The wait gives up,
 * FDS_STATUS_TMA_TIMEOUT is ORed into *status (device int32) and the kernel returns;
 * no copy is left in flight. Tests the timeout path end to end without a fault.
 * No counterpart in the reference (pyfds has no GPU and no bounded waits).
 */
int32_t fds_selftest_bounded_wait(int32_t mode, int32_t* status, const uint32_t* counter,
                                  int64_t poll_limit, void* stream);

/* Size of the scratch array built into the library for fds_stag_batch_run_static. */
#define FDS_BATCH_STATIC_MAX_BYTES (8u << 20)

/*
 * fds_stag_batch_run without a caller-allocated workspace: the same batched run
 * (upload and launch), with its descriptors and work list in a scratch array of
 * FDS_BATCH_STATIC_MAX_BYTES compiled into this library. It allocates no device
 * memory, for callers that cannot allocate (a C or Fortran host code with no
 * device allocator of its own, or a section where an allocation is not allowed).
 * No counterpart in the reference (pyfds has no GPU and no C interface).
 * - A batch whose workspace (fds_stag_batch_workspace_bytes) exceeds the maximum
 *   is rejected with FDS_E_SIZE.
 * - Every call looks up the array's device address on the current device
 *   (cudaGetSymbolAddress, no allocation), so the address stays right after a
 *   device reset. The first call on a device also loads the module: make it
 *   before any stream capture.
 * - A call whose stream is capturing is rejected with FDS_E_ARG (the call copies
 *   its descriptors from host memory that it frees on return).
 * - Every call shares the one array: calls whose work overlaps on the GPU (other
 *   streams, other threads) race and must be serialised by the caller.
 */
int32_t fds_stag_batch_run_static(const FdsStagProblem* probs, FdsStagState* states,
                                  const FdsStagTables* tables, int32_t count, int64_t step0,
                                  int32_t nsteps, int32_t store_flux, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FDS_CAPI_H */
