/*
 * bookleaf_gb300.h -- C-ABI of the GB300 (sm_103a) hydro hot path.
 *
 * This library replaces BookLeaf's per-step solver entry points
 *   inf_solver_getdt   (src/infrastructure/solver/inf_solver_getdt.f90:35-70)
 *   inf_solver_lagstep (src/infrastructure/solver/inf_solver_lagstep.f90:44-78)
 *   inf_solver_alestep (src/infrastructure/solver/inf_solver_alestep.f90:39-74)
 * for a single-partition mesh.  The caller owns every field array for the
 * whole run, exactly as BookLeaf's data_t handles do
 * (src/dataAPI/dataAPI_types.f90:31-38, src/utilities/data/data.f90:129-304);
 * the library keeps device mirrors and copies back on request.
 *
 * Conventions (all taken from the reference):
 *  - Arrays are registered through a table of host pointers indexed by the
 *    reference's dataAPI field IDs (src/dataAPI/dataAPI_id.f90:26-74), so a
 *    Fortran host passes C_LOC(dh(id)%raddr(1)) / C_LOC(dh(id)%iaddr(1)).
 *  - Corner and face arrays are Fortran (NCORN,nel) blocks: the four values
 *    of one element are contiguous.
 *  - Connectivity values are 1-based, as the Fortran host stores them.
 *  - Every entry point returns error%ierr and fills bl_error like
 *    error_t{ierr,iout,serr} (src/dataAPI/dataAPI_types.f90:76-79) with
 *    SUCCESS=0, FAILURE=-1, HALT_ALL=1, HALT_SINGLE=2
 *    (src/dataAPI/dataAPI_params.f90:31-34).  A negative volume returns
 *    ierr = -iel of the offending element (geometry_kn_volume.f90:81-99).
 *
 * Nothing in these signatures is a torch or CUDA type: plain pointers,
 * sizes and POD structs only.
 */
#ifndef BOOKLEAF_GB300_H
#define BOOKLEAF_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- dataAPI field IDs (src/dataAPI/dataAPI_id.f90:26-74) ---------------- */
enum {
  BL_ELDENSITY = 1, BL_ELENERGY = 2, BL_ELPRESSURE = 3, BL_ELCS2 = 4,
  BL_ELVOLUME = 5, BL_A1 = 6, BL_A2 = 7, BL_A3 = 8, BL_B1 = 9, BL_B2 = 10,
  BL_B3 = 11, BL_CNWT = 12, BL_CNX = 13, BL_CNY = 14,
  BL_RSCRATCH21 = 15, BL_RSCRATCH22 = 16, BL_RSCRATCH23 = 17,
  BL_RSCRATCH24 = 18, BL_RSCRATCH25 = 19, BL_RSCRATCH26 = 20,
  BL_RSCRATCH27 = 21, BL_RSCRATCH28 = 22,
  BL_CNVISCX = 23, BL_CNVISCY = 24, BL_ELVISC = 25, BL_ELMASS = 26,
  BL_CNMASS = 27,
  BL_RSCRATCH11 = 28, BL_RSCRATCH12 = 29, BL_RSCRATCH13 = 30,
  BL_RSCRATCH14 = 31, BL_RSCRATCH15 = 32, BL_RSCRATCH16 = 33,
  BL_RSCRATCH17 = 34,
  BL_NDX = 35, BL_NDY = 36, BL_NDU = 37, BL_NDV = 38, BL_INDTYPE = 39,
  BL_IELSORT1 = 40, BL_IELND = 41, BL_IELEL = 42, BL_IELFC = 43,
  BL_IELMAT = 44, BL_IELREG = 45, BL_IELSORT2 = 46, BL_SPMASS = 47,
  BL_ISCRATCH11 = 48, BL_ZSCRATCH11 = 49, BL_IELLOCGLOB = 50,
  BL_INDLOCGLOB = 51,
  BL_CPDENSITY = 52, BL_CPENERGY = 53, BL_CPPRESSURE = 54, BL_CPCS2 = 55,
  BL_CPVOLUME = 56, BL_FRVOLUME = 57, BL_CPMASS = 58, BL_FRMASS = 59,
  BL_CPVISCX = 60, BL_CPVISCY = 61, BL_CPVISC = 62, BL_CPA1 = 63,
  BL_CPA3 = 64, BL_CPB1 = 65, BL_CPB3 = 66, BL_ICPMAT = 67,
  BL_ICPNEXT = 68, BL_ICPPREV = 69, BL_IMXEL = 70, BL_IMXFCP = 71,
  BL_IMXNCP = 72, BL_ICPSCRATCH11 = 73, BL_ICPSCRATCH12 = 74,
  BL_RCPSCRATCH11 = 75, BL_RCPSCRATCH21 = 76, BL_RCPSCRATCH22 = 77,
  BL_RCPSCRATCH23 = 78, BL_RCPSCRATCH24 = 79,
  BL_NID = 79
};

/* error_t codes (src/dataAPI/dataAPI_params.f90:31-34) */
enum { BL_SUCCESS = 0, BL_FAILURE = -1, BL_HALT_ALL = 1, BL_HALT_SINGLE = 2 };

/* Maximum materials / regions accepted (the reference's namelist bound LN). */
#define BL_MAXMAT 100
#define BL_MAXREG 100
#define BL_NEOSPARAM 6
#define BL_SLEN 130

/* sizes_t (src/dataAPI/dataAPI_types.f90:40-43).  nel1=nel2=nel and
 * nnd1=nnd2=nnd for one partition (init_kn.f90:108-119). */
typedef struct {
  int nel, nel1, nel2, nnd, nnd1, nnd2, nsz, nmat, nreg, ncp, nmx, mcp, mmx;
} bl_sizes;

/* The configuration scalars the hot path reads, flattened from config_t:
 *   time_t   src/packages/time/config/time_types.f90:26-32
 *   hydro_t  src/packages/hydro/config/hydro_types.f90:28-39
 *   global_t src/utilities/data/global_types.f90 (zcut,zerocut,dencut,accut)
 *   eos_t    src/utilities/eos/config/eos_types.f90:24-28, already
 *            rationalised to materials 0..nmat (eos_config.f90:163-226)
 *   ale_t    src/packages/ale/config/ale_types.f90:27-42
 * Per-region arrays are indexed 0..nreg-1 for regions 1..nreg.  The EoS
 * tables are indexed by material 0..nmat (material 0 = void). */
typedef struct {
  /* time_t */
  double time_start, time_end, dt_g, dt_min, dt_max, dt_initial;
  /* hydro_t */
  double cvisc1, cvisc2, cfl_sf, div_sf;
  int ztq, zhg, zsp, pad0;
  double kappareg[BL_MAXREG], pmeritreg[BL_MAXREG];
  int zdtnotreg[BL_MAXREG], zmidlength[BL_MAXREG];
  /* global_t */
  double zcut, zerocut, dencut, accut;
  /* eos_t */
  double ccut, pcut;
  int eos_type[BL_MAXMAT + 1];
  int pad1;
  double eos_param[BL_MAXMAT + 1][BL_NEOSPARAM];
  /* ale_t */
  int ale_zexist, ale_zon, ale_zeul, ale_adv_type, ale_npatch, pad2;
  double ale_mintime, ale_maxtime, ale_sf;
} bl_config;

/* timestep_t (src/dataAPI/dataAPI_types.f90:45-51).  mdt is reported as the
 * material number imdt of the controlling element (>0), 0 for a mixed cell
 * and -1 for none, because the library does not hold material names. */
typedef struct {
  double time, dt, dts;
  int nstep, idtel, zcorrector, imdt;
  char sdt[9];
  char mdt[11];
} bl_timestep;

/* error_t (src/dataAPI/dataAPI_types.f90:76-79) */
typedef struct {
  int ierr, iout;
  char serr[BL_SLEN + 1];
} bl_error;

/* Floating-point modes.  BL_FP_EXACT evaluates every expression in the
 * reference's order without fused multiply-add, which reproduces a
 * -ffp-contract=off CPU build bit for bit.  BL_FP_FAST lets the compiler
 * contract a*b+c into one FMA (gfortran does the same at -O2 on aarch64);
 * results then differ from the CPU build in the last bits.  BL_FP_MIXED
 * (no counterpart in the reference: the demoted form for batches) is
 * BL_FP_FAST with the edge viscosity's limiter ratios, edge coefficients
 * and edge forces, the CFL lengths and divergence, and the remap limiters'
 * gradients in FP32; positions, geometry and volumes, pressure forces,
 * the energy update, the remap fluxes and the dt reduction stay FP64.
 * Other values are rejected. */
enum { BL_FP_FAST = 0, BL_FP_EXACT = 1, BL_FP_MIXED = 2 };

typedef struct bl_ctx bl_ctx;

/* One row of the dt history written by bl_run (time_dr_end's mindt,
 * src/packages/time/driver/time_dr_advance.f90:89-119). */
typedef struct {
  double time, dt;
  int nstep, idtel, sdt_code, ierr;
} bl_step_record;

/* sdt codes used in bl_step_record, in time_dr_calc/hydro_dr_getdt order. */
enum { BL_DT_MAXIMUM = 0, BL_DT_GROWTH = 1, BL_DT_INITIAL = 2, BL_DT_CFL = 3,
       BL_DT_DIV = 4 };

/* ---- lifetime ------------------------------------------------------------ */

/* Allocates device mirrors and uploads every registered field.  Replaces the
 * state the reference builds in inf_init (src/infrastructure/init/
 * inf_init.F90:53-103): the caller has already generated the mesh, the
 * connectivity ielel/ielfc, the node types, the initial state, the masses
 * and (if zsp) spmass.  dh has BL_NID+1 entries; dh[0] is unused and dh[id]
 * is the host array of field id (NULL for fields the path does not need:
 * scratch, component arrays when ncp==0, spmass when zsp is false,
 * ielsort2 when there is no ALE).  fp_mode is BL_FP_FAST, BL_FP_EXACT or
 * BL_FP_MIXED.  The device ordinal is the current CUDA device of the
 * calling thread.  The connectivity is checked on the device before any
 * kernel indexes with it; a bad table returns BL_FAILURE with HALT_ALL and,
 * in this order of precedence, "connectivity out of range" (ielnd, ielel,
 * ielfc), "ielreg/ielsort1 out of range", "ielsort1 is not a permutation",
 * "ielmat out of range", then the host's checks of ielsort2 and the
 * mixed-cell lists. */
int bl_init(bl_ctx **ctx, const bl_sizes *sizes, const bl_config *config,
            void *const *dh, int fp_mode, bl_error *error);

/* Frees every device allocation of the context. */
int bl_finalize(bl_ctx *ctx);

/* ---- the three solver entry points ------------------------------------- */

/* inf_solver_getdt (inf_solver_getdt.f90:35-70): dt candidates
 * (time_dr_calc), edge viscosity, elcs2 += elvisc, CFL and divergence
 * limits, then time_dr_end (nstep+1, dt, time += dt, dt_min check).
 * timestep is INOUT like runtime%timestep. */
int bl_getdt(bl_ctx *ctx, bl_timestep *timestep, bl_error *error);

/* inf_solver_lagstep (inf_solver_lagstep.f90:44-78): predictor and
 * corrector.  Leaves timestep%zcorrector=1 and dts=dt like the reference. */
int bl_lagstep(bl_ctx *ctx, bl_timestep *timestep, bl_error *error);

/* inf_solver_alestep (inf_solver_alestep.f90:39-74): returns at once
 * unless ale_active; otherwise flux volumes, advection and the hydro
 * update (inf_solver_aleupdate.f90:34-56). */
int bl_alestep(bl_ctx *ctx, const bl_timestep *timestep, bl_error *error);

/* The reference's time loop (inf_control_solver.f90:53-69) run on the
 * device: up to max_steps of getdt+lagstep+alestep, stopping after the step
 * whose time reaches time_end (time_finish, time_dr_utils.f90:57-69) or on
 * the first error.  dt selection and the end test happen on the device and
 * the steps are replayed from CUDA graphs, so the host does not wait per
 * step.  history (may be NULL) receives one record per step taken;
 * *nsteps receives their number.  timestep is INOUT. */
int bl_run(bl_ctx *ctx, bl_timestep *timestep, int max_steps,
           bl_step_record *history, int *nsteps, bl_error *error);

/* ---- data movement ------------------------------------------------------- */

/* Copies device field id back into the host array registered for it (the
 * reference's host readers: inf_io_output, check_dr_validate,
 * hydro_dr_shortprint).  id = 0 copies every registered state field. */
int bl_sync_to_host(bl_ctx *ctx, int id);

/* Uploads host field id again after the host changed it (id = 0: all). */
int bl_sync_to_device(bl_ctx *ctx, int id);

/* ---- batches of meshes (no counterpart in the reference) ------------------
 * Several independent problems -- each what one control file describes, with
 * its own mesh, materials, time-step controls and end time -- advanced
 * together: one kernel per phase over all of them, each mesh keeping its own
 * dt and time on the device.  The results of every mesh are those of running
 * it alone (bit for bit in BL_FP_EXACT).
 *
 * bl_init_batch: ninst meshes; sizes[i], configs[i] and the dataAPI table
 * dh[i] describe mesh i exactly as bl_init's arguments do (the same fields
 * registered for every mesh).  The hydro, cut-off and ALE settings must be
 * the same for all meshes; the time-step controls, regions and materials
 * may differ.  Mixed cells are not supported in a batch.  The solver entry
 * points, bl_run, bl_time_step_kernels and the diagnostics refuse a batch
 * context; bl_sync_to_host / bl_sync_to_device move every mesh's own arrays.
 *
 * bl_run_batch: advances all meshes on the device (graphs of 16 steps) from
 * ts[0..ninst-1] until each has reached its time_end or stopped on an error,
 * or max_steps steps have run (a mesh already at its time_end does not
 * advance); ts[i] receives mesh i's timestep, status[i]
 * (may be NULL) its error%ierr (0, -1, or -iel of a negative volume), and
 * *nsteps the number of steps run.  Returns BL_SUCCESS when no mesh failed,
 * else BL_FAILURE with err naming the first failed mesh. */
int bl_init_batch(bl_ctx **ctx, int ninst, const bl_sizes *sizes, const bl_config *configs,
                  void *const *const *dh, int fp_mode, bl_error *err);
int bl_run_batch(bl_ctx *ctx, bl_timestep *ts, int max_steps, int *status, int *nsteps,
                 bl_error *err);
/* Number of meshes of a batch context (0 for a single mesh). */
int bl_batch_size(bl_ctx *ctx);
/* The batch's autotuner: times each candidate of the steps per graph (8, 16,
 * 32) and the block size of the node kernels (128, 256, 512) over the same
 * 32 steps from ts, keeps the fastest for the following bl_run_batch calls
 * and reports it.  It runs from the state in the meshes' registered host
 * arrays and uploads that state again when done, so call it when those
 * arrays hold the state to run from (after bl_init_batch, or after
 * bl_sync_to_host).  ms_per_step[0..8] (may be NULL) receives each
 * candidate's time per step, G-major. */
int bl_autotune_batch(bl_ctx *ctx, const bl_timestep *ts, int *graph_steps, int *node_block,
                      double *ms_per_step, int n_ms, bl_error *err);

/* ---- the learned mixed-cell closure's network (no counterpart in the
 * reference) ----------------------------------------------------------------
 * A 10 -> 64 -> 64 -> 2 MLP with SiLU, trained and evaluated on the tensor
 * cores (BF16 operands, FP32 accumulation).  Parameters are FP32, laid out
 * W1[64][10], b1[64], W2[64][64], b2[64], W3[2][64], b3[2].  The loss is the
 * mean over samples of |y - t|^2 / 2.  All calls take host arrays (row per
 * sample) and return 0, or -1 when CUDA fails. */
#define BL_MLP_IN 10
#define BL_MLP_HIDDEN 64
#define BL_MLP_OUT 2
#define BL_MLP_NPARAM 4994
typedef struct bl_mlp bl_mlp;
int bl_mlp_create(bl_mlp **m, const float *params);
int bl_mlp_destroy(bl_mlp *m);
/* the current parameters */
int bl_mlp_params(bl_mlp *m, float *params);
/* y[n][2] for x[n][10] */
int bl_mlp_predict(bl_mlp *m, const float *x, int n, float *y);
/* the loss and its gradient with respect to the parameters over all n samples */
int bl_mlp_gradient(bl_mlp *m, const float *x, const float *t, int n, float *grad, float *loss);
/* Adam (lr, betas 0.9 / 0.999) over shuffled mini-batches (seeded);
 * losses[epochs] (may be NULL) receives each epoch's mean loss */
int bl_mlp_train(bl_mlp *m, const float *x, const float *t, int n, int epochs, int batch,
                 float lr, unsigned long long seed, float *losses);

/* The learned mixed-cell closure in a context's Lagrangian step (no
 * counterpart in the reference, whose closure keeps each material's volume
 * fraction through the step).  With on = 1, the network net (its current
 * parameters are copied: it may be trained further or destroyed after the
 * call) predicts, for every two-material mixed cell, the volume
 * each material gains over the step beyond its volume-fraction share, as a
 * fraction of the cell's volume, norm[20] * output, from ten features of
 * the cell at the start of the step standardised as (f - norm[k]) *
 * norm[10 + k]: material 1's volume fraction, the two densities, pressures
 * and sound speeds squared, dV / V, dt sqrt(max cs2 / V) and (p1 - p2) /
 * (|p1| + |p2|).  The exchange is limited to the range that moves the two
 * materials towards pressure equilibrium and not past it.  A cell whose
 * outputs are not finite, do not cancel within norm[21] (volume
 * conservation), lie farther outside that range than its width, or leave a
 * material a non-positive volume keeps the plain closure.  on = 1: the
 * exchanged volume trades energy at the mixture pressure (the work one
 * material does on the other); on = 2: the materials keep their specific
 * energies, so that for ideal gases the cell's mixture pressure, and with
 * it every element and node field of the run, stays the plain closure's.
 * Either way each cell's volume and total energy are the plain closure's.
 * on = 0 restores the plain closure everywhere.  On a batch context it
 * applies to every mesh. */
int bl_set_closure(bl_ctx *ctx, bl_mlp *net, const float *norm, int on, bl_error *err);
/* cells the closure has seen and cells it handed back to the plain closure */
int bl_closure_stats(bl_ctx *ctx, unsigned long long *cells, unsigned long long *rejected);

/* ---- introspection ------------------------------------------------------- */

/* Waits for the context's stream.  Returns 0 or a CUDA error number. */
int bl_synchronize(bl_ctx *ctx);

/* The cudaStream_t the context launches on, as an opaque pointer, for
 * callers that time or order work against it. */
void *bl_stream(bl_ctx *ctx);

/* Number of kernels this context has launched so far. */
long long bl_kernel_launches(bl_ctx *ctx);

/* Durations of the kernels of a Lagrangian step at the context's current
 * state (no counterpart in the reference; a measurement aid).  Advances
 * the state by nstep steps (1..64) from *ts: the kernels of the getdt and
 * lagstep entry points are queued back to back on the context's stream
 * with a CUDA event between each and no host copy between steps, without
 * the end-time stop of bl_run (so it also runs past time_end).  ms[0..3]
 * (n >= 4) receive the mean durations in milliseconds of the getdt
 * kernel and of the three lagstep kernels (force, acceleration, state);
 * *ts receives the state after the last step.  The ALE step is not run.
 * Returns BL_SUCCESS, or BL_FAILURE with *err set as the solver entry
 * points set it. */
int bl_time_step_kernels(bl_ctx *ctx, bl_timestep *ts, int nstep, double *ms, int n,
                         bl_error *err);

/* Library version string. */
const char *bl_version(void);

/* Self-test of the integer-pipe FP64 arithmetic the kernels use in place of
 * the hardware divide and square root (no counterpart in the reference): n
 * operands (random, plus hard cases) are computed both ways on the current
 * device; *mismatches receives the number of results that differ in any
 * bit, first_a/first_b the first failing operands.  op 0: division a/b;
 * op 1: square root of a; op 2: product a*b.  Returns 0, or -1 when CUDA
 * fails. */
int bl_selftest_fp64(int op, long long n, unsigned long long seed, long long *mismatches,
                     double *first_a, double *first_b);

/* Issue rates on the current device, in G operations/s (no counterpart in
 * the reference): rates[0] FP64 FMA, [1] hardware divide, [2] integer-pipe
 * divide, [3] hardware square root, [4] integer-pipe square root, and when
 * n >= 7 [5] hardware multiply, [6] integer-pipe multiply.  n >= 5.
 * The FMA rate is the FP64 roof the hot path's kernels are measured
 * against.  Returns 0, or -1 when CUDA fails. */
int bl_fp64_rates(double *rates, int n);

/* ---- diagnostics on the device ------------------------------------------ */

/* Columns of one bl_shortprint row. */
#define BL_SP_NQ 10

/* hydro_dr_shortprint's reductions (src/packages/hydro/driver/
 * hydro_dr_print.f90:49-170) from the device state, for a host that prints
 * the short print without copying the fields back: table 0 per region,
 * table 1 per material (mixed-cell components included, as
 * utils_kn_mxgathercncp feeds them).  out receives nflag rows (nflag >=
 * nreg resp. nmat) of BL_SP_NQ values: volume, mass, internal energy,
 * kinetic energy, pressure (mass-weighted mean), minimum and maximum
 * pressure, density (mass/volume), minimum and maximum density.  The sums
 * are fixed trees, reproducible run to run; they differ from the
 * reference's serial sums in rounding only. */
int bl_shortprint(bl_ctx *ctx, int table, double *out, int nflag, bl_error *error);

/* check_dr_sod (src/packages/check/driver/check_dr_tests.f90:34-71) on the
 * device: L1 norms of density and energy against the exact Sod solution in
 * the reference check's geometry (interface at x = 50, gamma 1.4). */
int bl_check_sod(bl_ctx *ctx, double time, double *l1_density, double *l1_energy,
                 bl_error *error);

/* ---- allocation-free getdt ---------------------------------------------- */

/* Largest mesh bl_getdt_noalloc accepts: its reduction scratch lives in a
 * fixed 1.5 MiB device array (65,536 blocks of 128 elements). */
#define BL_NOALLOC_MAX_NEL (65536 * 128)

/* Device arrays for bl_getdt_noalloc, in the reference's own layout: every
 * pointer is device memory the caller owns; connectivity is 1-based;
 * corner/face arrays are (NCORN,nel) blocks.  Pure-material meshes only
 * (no mixed cells). */
typedef struct {
  int nel, nnd;
  const double *ndx, *ndy, *ndu, *ndv;           /* [nnd] */
  const int *indtype;                            /* [nnd] */
  const int *ielnd, *ielel, *ielfc;              /* [4*nel], 1-based */
  const int *ielreg;                             /* [nel], 1-based */
  const double *eldensity, *elcs2;               /* [nel] inputs */
  const double *a1, *a3, *b1, *b3, *elvolume;    /* [nel] inputs */
  double *cnviscx, *cnviscy;                     /* [4*nel] outputs */
  double *elvisc;                                /* [nel] output */
  double *elcs2_out;                             /* [nel] output: elcs2+elvisc */
} bl_getdt_arrays;

/* No counterpart in the reference: an allocation-free variant of bl_getdt
 * for callers that cannot call cudaMalloc -- for example a host that hands
 * out every byte of device memory from its own pool, so that a library
 * allocating behind its back would fail or break its accounting.  It runs
 * bl_getdt's computation (edge viscosity, elcs2+elvisc, CFL and divergence
 * limits, time_dr_calc/time_dr_end) on arrays the caller passes, without a
 * bl_ctx: the library's own exact-form getdt kernel, so its results equal
 * bl_getdt's in BL_FP_EXACT mode bit for bit.  Its reduction scratch is a fixed file-scope device
 * array, held by every GPU that loads the library until the process exits;
 * nothing is allocated or freed by this call.  The first call on a device
 * looks up that array's device address (cudaGetSymbolAddress); make that
 * first call before any stream capture.  Calls that overlap on the GPU
 * (other streams, other host threads) share the array and race: serialise
 * them.  elcs2_out must not alias elcs2 (neighbouring elements read elcs2
 * while it is written), and every ielreg entry must lie in 1..BL_MAXREG
 * (entries outside it read region 1's settings).
 * Returns the reference's error codes like bl_getdt; nel >
 * BL_NOALLOC_MAX_NEL is rejected with FAILURE.  stream is a cudaStream_t
 * (NULL: the legacy default stream); the call copies the result record to
 * the host and synchronises that stream before it returns timestep. */
int bl_getdt_noalloc(const bl_getdt_arrays *arrays, const bl_config *config,
                     bl_timestep *timestep, void *stream, bl_error *error);

#ifdef __cplusplus
}
#endif

#endif /* BOOKLEAF_GB300_H */
