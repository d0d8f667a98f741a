/*
 * fdp.h -- C ABI of the GB300 time-stepping engine for the 2-D
 * velocity-stress Biot poroelastic finite-difference simulator
 * (drop-in for the TIME_LOOP body of David011/2D-VQSP-FD-Sim).
 *
 * The reference has no plugin or FFI API: its seam is the TIME_LOOP
 * subroutine (time_loop.F90:3-209) and the module state it USEs
 * (WAVEFIELD, STRESSFIELD, GRID_MEDIUM, PML, NONREF_BOUND, AUXIL,
 * CONTROL_DATA).  Each entry point below replaces one piece of that
 * seam; the comment on each names the reference code it stands in for.
 *
 * Conventions
 *   - Every function returns FDP_OK (0) on success or a negative FDP_ERR_*
 *     code; fdp_last_error() gives a one-line message.  Nothing throws.
 *   - Host arrays use the reference's Fortran layout: column-major, x
 *     fastest, with the Fortran lower bounds stated per argument (PMLL =
 *     1-TPML may be negative, rows start at 0).  No transposition is needed
 *     by a Fortran caller.
 *   - Real-valued host arrays are in the precision selected at fdp_create
 *     (FDP_F32 = REAL(4), FDP_F64 = REAL(8)); that is the reference's
 *     working precision PP (mod_precision.F90:7,10).
 *   - The context owns all device memory; the caller owns all host memory.
 *   - One host thread per context; one CUDA stream per context (its frame
 *     kernels run on a second stream forked from and joined back into it;
 *     fdp_get_stream returns the first).  fdp_run only enqueues work;
 *     fdp_get_* and fdp_synchronize wait for it.
 */
#ifndef FDP_H
#define FDP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FDP_OK 0
#define FDP_ERR_ARG (-1)         /* invalid argument or unsupported geometry   */
#define FDP_ERR_CUDA (-2)        /* a CUDA runtime call failed                 */
#define FDP_ERR_ALLOC (-3)       /* device or host allocation failed           */
#define FDP_ERR_STATE (-4)       /* call out of order (e.g. run before set_*)  */
#define FDP_ERR_UNSUPPORTED (-5) /* field not held by this engine              */
#define FDP_ERR_DEVICE (-6)      /* a kernel reported that a bounded wait expired */

#define FDP_F32 4
#define FDP_F64 8

/* Grid and control data.  Mirrors CONTROL_DATA/AUXIL after READ_OPEN and
 * AUX1 (read_open.F90:144-171, aux1.F90:36-46): mz is the value after the
 * stress-imaging shift MZ=MZ+2 (read_open.F90:149-151) and lin_z the source
 * row after the +2H shift (read_open.F90:165-169). */
typedef struct fdp_grid {
  int32_t mx, mz;          /* MX, MZ                                          */
  int32_t tpml;            /* TPML, PML thickness in cells                    */
  int32_t stress_imaging;  /* STRESS_IMAGING (1) or one-sided free surface (0) */
  int32_t lin_x, lin_z;    /* source cell LIN_X, LIN_Z                        */
  int32_t precision;       /* FDP_F32 or FDP_F64                              */
  int32_t device;          /* CUDA device ordinal                             */
  double h, dt, tau_eps;   /* H, DT, TAU_EPS (READ_OPEN forces TAU_EPS=0)     */
} fdp_grid;

typedef struct fdp_ctx fdp_ctx;

/* Field identifiers for fdp_get_field / fdp_set_field / fdp_field_bounds.
 * Bounds are those of the reference's arrays (ppml.F90:85-112,
 * tl_alloc.F90:24-36, alloc_nr.F90:33-40). */
enum fdp_field_id {
  FDP_UM = 0, FDP_WM, FDP_QX, FDP_QZ, FDP_TXX, FDP_TZZ, FDP_TXZ, FDP_PRES,
  FDP_PZXL, FDP_PZXH, FDP_PXXL, FDP_PXXH, FDP_OXXL, FDP_OXXH, FDP_PXZH, FDP_PZZH, FDP_OZZH,
  FDP_RXXL, FDP_RXXH, FDP_SXXL, FDP_SXXH, FDP_RZXL, FDP_RZXH, FDP_GXXL, FDP_GXXH,
  FDP_HXXL, FDP_HXXH, FDP_GZXL, FDP_GZXH, FDP_RXZH, FDP_GXZH, FDP_RZZH, FDP_SZZH,
  FDP_GZZH, FDP_HZZH,
  /* bottom-row history SZ_U/SZ_W/SZ_QX/SZ_QZ (mod_nr_bound.F90:43-47) as
   * (PMLL:PMLXH, 0:2), row k holding component TIKMZk */
  FDP_SZ_U, FDP_SZ_W, FDP_SZ_QX, FDP_SZ_QZ,
  /* QXP/QZP (old-q copies): not stored by this engine, which reads the
   * pre-update q at the same cell instead; get/set return FDP_ERR_UNSUPPORTED */
  FDP_QXP, FDP_QZP,
  FDP_FIELD_COUNT
};

/* Snapshot mask bits for fdp_get_snapshot. */
#define FDP_SNAP_UM (1 << 0)
#define FDP_SNAP_WM (1 << 1)
#define FDP_SNAP_QX (1 << 2)
#define FDP_SNAP_QZ (1 << 3)

/* Receiver flags for fdp_set_receivers (KEYS namelist, read_open.F90:52). */
#define FDP_REC_TLV (1 << 0) /* KEY_TLV: u, -w (store_seismograms.F90)        */
#define FDP_REC_TLQ (1 << 1) /* KEY_TLQ: qx, -qz                              */
#define FDP_REC_TLP (1 << 2) /* KEY_TLP: p, -txx (store_seismograms_pressure) */

/* Number of values per receiver per time level returned by
 * fdp_get_receivers, in this order:
 *   SSU SSW SPU SPW        (REC_UW_<j>.asc columns 2-5, store_seismograms.F90:144)
 *   SSQX SSQZ ZPU ZPW      (REC_Q_<j>.asc columns 2-5, store_seismograms.F90:150)
 *   SSP SST                (REC_STRESS_<j>.asc columns 2-3, store_seismograms_pressure.F90:80) */
#define FDP_REC_VALUES 10

/* Creates a context and allocates the device state, zeroed as TL_ALLOC,
 * PPML and ALLOC_NR do (tl_alloc.F90:44-56, ppml.F90:115-153,
 * alloc_nr.F90:42-54).  Replaces the allocations of TL_ALLOC/PPML/ALLOC_NR.
 * The environment variable FDP_KERNEL_VARIANT, read here, selects the
 * kernels, all bit-identical.  Unset: FP32 contexts whose levels outgrow
 * one and a half times the L2 cache run both phases of each level's deep
 * interior in one pass (fdp_march_info), every other context the split; "march" runs them so
 * on any grid large enough for the pass.
 * "split": the interior ("core") of each phase runs vectorised beside a
 * frame kernel for the PML, free-surface, source and bottom cells on a
 * second stream; "fused" runs frame and core of a phase in one launch;
 * "global" runs one unit kernel per phase over the whole grid; "tma" the
 * TMA-staged variant of the latter; "coretma" the split with TMA-staged
 * persistent core kernels (FP32 contexts with a Biot-plane medium; others
 * keep the per-thread-load core). */
int fdp_create(const fdp_grid* grid, fdp_ctx** out);

/* Medium: JM(PMLL:PMLXH, 0:PMLZH) (nx = MX+2*TPML, nz = PMLZH+1) after
 * READ_MODEL's row/column replication (read_model.F90:57-89), and the
 * material table as READ_MODEL_PAR holds it after scaling
 * (read_model_par.F90:52-74): table24[(jm-1)*24 + k], k in the .MO record
 * order MU SIG_XX_1..3 SIG_ZZ_1..3 PRES_1..3 REL1_U REL1_W REL2_U REL2_W
 * REL3_U REL3_W REL1_QX REL1_QZ REL2_QX REL2_QZ REL3_QX REL3_QZ AUXIL_W
 * AUXIL_QZ, REL* already multiplied by DT and divided by H as
 * read_model_par.F90:63-74 does. */
int fdp_set_medium(fdp_ctx* ctx, const int32_t* jm, int32_t nx, int32_t nz, int32_t jmnum,
                   const void* table24);

/* Makes dst use src's device medium (JM, material table or per-cell planes,
 * AUXIL) instead of holding its own copy: shots of one survey over the same
 * model (GRID_MEDIUM is the same module state for all of them in the
 * reference, read_model.F90 / read_model_par.F90) keep one copy in HBM and
 * derive it once.  Both contexts need the same grid (MX, MZ, TPML),
 * precision and device, and src a medium.  dst's own medium is freed; the
 * shared arrays live until the last context using them is destroyed or
 * given a medium of its own by fdp_set_medium. */
int fdp_share_medium(fdp_ctx* dst, fdp_ctx* src);

/* PML damping profiles from PPML (ppml.F90:156-306), 24 arrays in this order:
 *   ODA_XL ODB_XL ODC_XL ODD_XL ODA_XH ODB_XH ODC_XH ODD_XH      (0:TPML,   0:PMLZH)
 *   ODA_ZH ODB_ZH ODC_ZH ODD_ZH                                  (0:TPML,   PMLL:PMLXH)
 *   ODA2_XL ODB2_XL ODC2_XL ODD2_XL ODA2_XH ODB2_XH ODC2_XH ODD2_XH (0:TPML+1, 0:PMLZH)
 *   ODA2_ZH ODB2_ZH ODC2_ZH ODD2_ZH                              (0:TPML+1, PMLL:PMLXH) */
int fdp_set_pml(fdp_ctx* ctx, const void* const* profiles24);

/* The same 24 profiles as separate arguments, in the same order: the form a
 * Fortran caller binds, passing the PML module's arrays (ALLOCATABLE,
 * mod_pml.F90:7-15) by reference as assumed-size dummies, since taking
 * their C address would need the TARGET attribute they lack. */
int fdp_set_pml_arrays(fdp_ctx* ctx, const void* oda_xl, const void* odb_xl, const void* odc_xl,
                       const void* odd_xl, const void* oda_xh, const void* odb_xh, const void* odc_xh,
                       const void* odd_xh, const void* oda_zh, const void* odb_zh, const void* odc_zh,
                       const void* odd_zh, const void* oda2_xl, const void* odb2_xl, const void* odc2_xl,
                       const void* odd2_xl, const void* oda2_xh, const void* odb2_xh, const void* odc2_xh,
                       const void* odd2_xh, const void* oda2_zh, const void* odb2_zh, const void* odc2_zh,
                       const void* odd2_zh);

/* Bottom non-reflecting coefficients from PRE_NR_COEF1 (pre_nr_coef1.F90:187-202):
 * ABW01 ABW02 ABW10 ABW11 ABW12 ABW20 ABW21 ABW22 ABH01 ... ABH22. */
int fdp_set_bottom_nr(fdp_ctx* ctx, const void* ab16);

/* Source time function SOURTF_A(2, MT2) (open_sr_file.F90:41-110), column-major:
 * sourtf[2*(it-1)] = solid part, sourtf[2*(it-1)+1] = fluid part. */
int fdp_set_source(fdp_ctx* ctx, const void* sourtf, int32_t mt2);

/* Receivers IRECX, LRECX, IRECZ, LRECZ (read_open.F90:225-236) and the
 * FDP_REC_* flags (KEY_TLV/KEY_TLQ/KEY_TLP).  Replaces the sampling part of
 * STORE_SEISMOGRAMS / STORE_SEISMOGRAMS_PRESSURE. */
int fdp_set_receivers(fdp_ctx* ctx, const int32_t* irecx, const int32_t* lrecx, const int32_t* irecz,
                      const int32_t* lrecz, int32_t mr, int32_t flags);

/* Advances time levels it_begin..it_end (1-based, inclusive, it_end <= MT2):
 * the body of DO ITILE = MT1, MT2 (time_loop.F90:65-206) without its file
 * output.  Asynchronous: the levels are replayed from captured CUDA graphs
 * (see fdp_prepare_run). */
int fdp_run(fdp_ctx* ctx, int32_t it_begin, int32_t it_end);

/* Captures, without running anything, the CUDA graphs that a run of
 * n_levels levels replays: fdp_run replays one graph of 32 levels per 32
 * levels and one graph of the remaining levels, each captured on its first
 * use (and again after a set_* call changes the device parameters).  A
 * caller that times its runs, or whose first run must not pay for the
 * capture, calls this beforehand.  With march levels, whose runs of odd
 * length end in the other buffers, the graphs of both buffers are
 * captured.  No counterpart in the reference. */
int fdp_prepare_run(fdp_ctx* ctx, int32_t n_levels);

/* Copies receiver values of levels it_first..it_first+n_levels-1 (already
 * run) to host: n_levels * MR * FDP_REC_VALUES values, level-major.  The
 * values are exactly what STORE_SEISMOGRAMS(_PRESSURE) write in a serial
 * build; columns of a disabled flag are zero. */
int fdp_get_receivers(fdp_ctx* ctx, int32_t it_first, int32_t n_levels, void* host);

/* Copies the current wavefield to host for snapshots (store_snapshots.F90:173-190):
 * for each bit set in field_mask, in the order UM WM QX QZ, one
 * (PMLL:PMLXH, 0:PMLZH) column-major array. */
int fdp_get_snapshot(fdp_ctx* ctx, int32_t field_mask, void* host);

/* Full-state access (checkpoint/resume and testing): bounds of a field as
 * {lx, ux, lz, uz}, and copies of it in that Fortran layout. */
int fdp_field_bounds(fdp_ctx* ctx, int32_t id, int32_t* bounds4);
int fdp_get_field(fdp_ctx* ctx, int32_t id, void* host);
int fdp_set_field(fdp_ctx* ctx, int32_t id, const void* host);

/* Diagnostics of the failure path: enqueues a kernel that waits, at most
 * `polls` polls about 100 ns apart (1..2^20), for a device word nothing
 * sets, and then records the expired wait in the context's status word, as
 * a TMA-staged kernel does when its tile copy never arrives.  The next
 * fdp_synchronize (or fdp_get_*) returns FDP_ERR_DEVICE once; the status
 * word is then cleared and the context stays usable. */
int fdp_diag_wait_timeout(fdp_ctx* ctx, int32_t polls);

/* Waits for all work of the context. */
int fdp_synchronize(fdp_ctx* ctx);

/* The context's CUDA stream (a cudaStream_t), so a caller can order its own
 * work, or record its own events, after the engine's. */
int fdp_get_stream(fdp_ctx* ctx, void** stream);

/* Diagnostics: advances levels it_begin..it_end like fdp_run but without
 * graphs, with CUDA events around each part of a level (all levels are
 * enqueued before one wait, so the windows hold device time, not host
 * launch latency), and returns
 * the summed device time in milliseconds in ms_out[0..4] and the number of
 * timed launches in launches_out[0..4]: {stress phase, velocity phase,
 * row 1 and receivers (and an attached learned edge), stress core kernel,
 * velocity core kernel}.  A phase is its frame and core kernels together
 * (one kernel with FDP_KERNEL_VARIANT=global or tma, when the core entries
 * stay 0). */
int fdp_profile_run(fdp_ctx* ctx, int32_t it_begin, int32_t it_end, double* ms_out, int64_t* launches_out);

/* Number of CUDA kernel launches this context has enqueued since creation
 * (graph-launched kernels counted individually). */
int64_t fdp_kernel_launches(fdp_ctx* ctx);

/* How the medium is held on the device after fdp_set_medium: *mode is 0
 * when the kernels index the material table through JM, 1 when each
 * distinct coefficient column is a per-cell plane (columns equal up to sign
 * share a plane, constant columns need none), 2 when those planes are the
 * ten of an isotropic Biot medium (lambda+2mu in SIG_XX_1 and SIG_ZZ_2,
 * lambda in SIG_XX_2 and SIG_ZZ_1, alpha*M in SIG_XX_3, SIG_ZZ_3 and
 * -PRES_1, -PRES_2, the same relaxation columns for x and z, REL1_Q equal
 * to REL3_U), so the kernels resolve the aliases at compile
 * time; *planes_stress and *planes_velocity count the planes each phase
 * reads per cell. */
int fdp_medium_info(fdp_ctx* ctx, int32_t* mode, int32_t* planes_stress, int32_t* planes_velocity);

/* Core rectangles of the frame/core split: rect[0..3] = stress core
 * columns [x0, x1) and rows [z0, z1) (the source row excluded), rect[4..7]
 * the velocity core; zeros when the context runs other kernels. */
int fdp_core_info(fdp_ctx* ctx, int32_t* rect8);

/* The march levels (by default for FP32 contexts on grids whose levels
 * outgrow one and a half times the L2 cache): each level's deep
 * interior in one kernel pass (stress phase, then velocity phase, from
 * bands of rows staged in shared memory by bulk tensor copies), the levels
 * alternating between two buffers of each wavefield array, with the frame
 * kernels on the side stream.  region8 = the columns [x0, x1) and rows
 * [z0, z1) the march kernel updates, then those where it writes the new
 * stresses (the frame kernels write a band along the edges); shape4 =
 * strips of 30 four-cell vectors across, rows per band, CTAs of the
 * launch, warps per CTA.  All zero when the context's levels do not run as
 * march levels (another variant, FP64, a grid too small, a batch's
 * work-queue kernels or an attached learned edge holding it).  The launch
 * shape is chosen when the medium is set; environment
 * variables read then override it, for measurements and tests:
 * FDP_MARCH_ROWS (4, 6 or 8 rows per band), FDP_MARCH_CTAS (that many
 * CTAs, the strips' rows split evenly among them) and FDP_MARCH_SMS (plan
 * for that many SMs).  No counterpart in the reference (a kernel
 * arrangement of time_loop.F90:93-179). */
int fdp_march_info(fdp_ctx* ctx, int32_t* region8, int32_t* shape4);

/* Last error message of the context (or of the last failed call that has
 * no context -- fdp_create, fdp_receivers_noalloc -- when ctx is NULL). */
const char* fdp_last_error(const fdp_ctx* ctx);

/* Receiver capacity of fdp_receivers_noalloc. */
#define FDP_NOALLOC_MAX_RECEIVERS 16384

/* Receiver sampling that allocates no device memory.  It has no
 * counterpart in the reference.  It serves callers that cannot call
 * cudaMalloc: a host whose device arrays come from a memory pool it manages
 * itself, or a runtime that forbids allocation once it is running.  All
 * inputs and outputs are the caller's device memory:
 *   um wm qx qz pres txx  the wavefield after a completed level, each
 *                         (pmll:pmll+nx-1, 0:nz-1) column-major with leading
 *                         dimension ld elements, in precision `precision`;
 *   rec                   4*mr int32 (IRECX LRECX IRECZ LRECZ per receiver);
 *   out                   mr*FDP_REC_VALUES values, written exactly as one
 *                         level of fdp_get_receivers (flags as there).
 * The previous sample of each receiver, which the time derivative needs
 * (store_seismograms.F90:65-66), is kept between calls in one static device
 * array of FDP_NOALLOC_MAX_RECEIVERS entries that every GPU loading the
 * library holds until exit; larger mr is rejected with FDP_ERR_ARG.  The
 * derivative columns of a call are taken against the samples the previous
 * call stored.  A call with level == 1 starts from zero samples, as the
 * reference does; later levels must follow in order, one call per level.  To
 * start at a level k > 1 (a resumed run), first call it with the wavefield
 * of level k-1 and discard that call's output: otherwise the first call's
 * derivative columns use whatever an earlier call left in the array.  All
 * calls share the array, so calls that overlap on the GPU race.  The first
 * call on a device looks up the array's device address (and again after a
 * reset of the device's context); make it before any stream capture.  A
 * call with mr == 0 only does that look-up and launches nothing.  The
 * kernel is enqueued on `stream` (a cudaStream_t, may be 0); errors are
 * returned and described by fdp_last_error(NULL). */
int fdp_receivers_noalloc(int32_t precision, const void* um, const void* wm, const void* qx, const void* qz,
                          const void* pres, const void* txx, int32_t nx, int32_t nz, int32_t ld, int32_t pmll,
                          const int32_t* rec, int32_t mr, int32_t flags, double dt, int32_t level, void* out,
                          void* stream);

/* Frees the context and all its device memory (the DEALLOCATEs the
 * reference leaves to program exit). */
void fdp_destroy(fdp_ctx* ctx);

/* ---------------------------------------------------------------------------
 * Batched shots.  No counterpart in the reference, which runs one shot per
 * job.  A batch advances many prepared contexts together: each level is one
 * launch per phase for the whole batch, over a work queue of (shot, tile)
 * items that persistent CTAs take round-robin, and runs of levels are
 * replayed from CUDA graphs.  Shots may differ in grid size, medium and
 * its device representation (fdp_medium_info), free-surface mode, source,
 * receivers and PML width; they must share precision and device.  Shots
 * are grouped by free-surface mode and medium representation, one launch
 * per phase per group.  Every shot's values are bit-identical to running it
 * alone with fdp_run. */
typedef struct fdp_batch fdp_batch;

/* Groups n contexts, each with medium, PML, bottom coefficients and source
 * set.  The contexts stay owned by the caller and must outlive the batch;
 * while it exists, run them only through it.  After fdp_batch_synchronize
 * their receivers, snapshots and fields are read with the fdp_get_* calls.
 * The batch copies each context's device parameters: a context given a new
 * medium, source, receivers or edge afterwards makes fdp_batch_run return
 * FDP_ERR_STATE (create the batch again). */
int fdp_batch_create(fdp_ctx* const* shots, int32_t n, fdp_batch** out);

/* Advances every shot over levels it_begin..it_end (within every shot's
 * MT2).  Asynchronous.  Unless a shape was set, the first run tunes the
 * tile shape on its own first levels (each candidate computes the same
 * values, so no level is wasted or altered) and keeps the fastest.  While
 * a batch runs, its shots' own streams carry work (the shots mode). */
int fdp_batch_run(fdp_batch* b, int32_t it_begin, int32_t it_end);

/* Tile shape of the work queue: units_per_item vertically adjacent units
 * (32 columns by 8 or 32 rows each) per item, and `waves` persistent CTAs
 * per resident CTA slot of the GPU (0: one CTA per item).  units_per_item
 * = FDP_BATCH_SHOTS runs instead every shot's own kernels (those fdp_run
 * launches) on the shot's own stream, all shots side by side in one CUDA
 * graph per 32 levels.  units_per_item = 0 asks the next run to tune again
 * (the tuner times the nine queue shapes on two levels each and, when the
 * run has 32 more levels, the shots mode on one graph of them). */
#define FDP_BATCH_SHOTS (-1)
int fdp_batch_set_shape(fdp_batch* b, int32_t units_per_item, int32_t waves);
int fdp_batch_get_shape(fdp_batch* b, int32_t* units_per_item, int32_t* waves);

/* Waits for the batch and reports a failed kernel of any shot. */
int fdp_batch_synchronize(fdp_batch* b);
int64_t fdp_batch_kernel_launches(fdp_batch* b);
int fdp_batch_get_stream(fdp_batch* b, void** stream);
/* Last error of the batch (of the last failed fdp_batch_create when NULL). */
const char* fdp_batch_last_error(const fdp_batch* b);
/* Frees the batch (not its contexts). */
void fdp_batch_destroy(fdp_batch* b);

#ifdef __cplusplus
}
#endif

#endif /* FDP_H */
