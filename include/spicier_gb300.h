/*
 * spicier_gb300.h — C ABI of the GB300 batched-sweep backend.
 *
 * This header is the drop-in boundary for Spicier's batched-sweep hot path.
 * Every entry point takes plain pointers and sizes, returns an int status
 * (SP_OK = 0, negative = error) and never aborts the process.
 *
 * Reference interfaces replaced (paths relative to the Spicier repository):
 *   BatchedLuSolver trait ........ crates/spicier-batched-sweep/src/solver.rs:107-135
 *   BatchedSolveResult ........... crates/spicier-batched-sweep/src/solver.rs:44-75
 *   GpuBatchConfig ............... crates/spicier-batched-sweep/src/solver.rs:15-40
 *   BackendType .................. crates/spicier-batched-sweep/src/solver.rs:79-92
 *   BatchedSweepError ............ crates/spicier-batched-sweep/src/error.rs:7-43
 *   CudaBatchedLuSolver::solve_batch crates/spicier-backend-cuda/src/batched_lu.rs:373-494
 *   ConvergenceCriteria .......... crates/spicier-solver/src/newton.rs:9-34
 *   Gmin/SourceSteppingParams .... crates/spicier-solver/src/newton.rs:173-231
 *   solve_newton_raphson ......... crates/spicier-solver/src/newton.rs:70-131 (batched here)
 *   hash RNG ..................... crates/spicier-batched-sweep/src/rng.rs:39-227
 *   SweepStatistics/Accumulator .. crates/spicier-batched-sweep/src/statistics.rs:35-160
 *   Histogram / YieldSpec ........ crates/spicier-batched-sweep/src/statistics.rs:205-386
 *   AdaptiveTransientParams ...... crates/spicier-solver/src/transient/types.rs:78-107
 *   GmresConfig .................. crates/spicier-solver/src/gmres/mod.rs:34-51
 *
 * Ownership: the caller owns every buffer passed in.  Functions suffixed
 * _device take device pointers and a cudaStream_t passed as void*; they
 * enqueue work and return without synchronising.  Functions without the
 * suffix take host pointers, copy in, compute, copy out and synchronise.
 *
 * Threading: an sp_ctx may be used from several host threads; each call
 * serialises on the context's internal lock (the reference trait is
 * Send + Sync).  Device-pointer calls run on the caller's stream.
 */
#ifndef SPICIER_GB300_H
#define SPICIER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------- */
/* Status codes: mirror of BatchedSweepError (error.rs:7-43).             */
/* ---------------------------------------------------------------------- */
enum sp_status {
    SP_OK = 0,
    SP_ERR_NO_BACKEND = -1,        /* NoBackendAvailable                  */
    SP_ERR_BACKEND_INIT = -2,      /* BackendInit(String)                 */
    SP_ERR_MEMORY_ALLOC = -3,      /* MemoryAlloc(String)                 */
    SP_ERR_TRANSFER = -4,          /* Transfer(String)                    */
    SP_ERR_INVALID_DIMENSION = -5, /* InvalidDimension(String)            */
    SP_ERR_BATCH_TOO_LARGE = -6,   /* BatchTooLarge { size, max }         */
    SP_ERR_SINGULAR_BATCH = -7,    /* SingularBatch (reserved)            */
    SP_ERR_BACKEND = -8,           /* Backend(String)                     */
    SP_ERR_SOLVER = -9,            /* Solver(spicier_solver::Error)       */
    SP_ERR_INVALID_ARGUMENT = -10  /* null pointer / bad enum value       */
};

/* BackendType (solver.rs:79-92) with one added tag for this backend. */
enum sp_backend_type {
    SP_BACKEND_CUDA = 0,
    SP_BACKEND_METAL = 1,
    SP_BACKEND_MPS = 2,
    SP_BACKEND_ACCELERATE = 3,
    SP_BACKEND_FAER = 4,
    SP_BACKEND_CPU = 5,
    SP_BACKEND_GB300 = 6
};

/* GpuBatchConfig (solver.rs:15-40).  Defaults here: min_batch_size 16,
 * min_matrix_size 1 (the fused kernels pay off from n = 1), and
 * max_batch_per_launch 1<<26 instead of the cuBLAS path's 65 535. */
typedef struct sp_batch_config {
    uint64_t min_batch_size;
    uint64_t min_matrix_size;
    uint64_t max_batch_per_launch;
} sp_batch_config;

/* Arithmetic used by a solve. */
enum sp_precision {
    SP_PREC_FP64 = 0,       /* plain FP64 everywhere (FMA contraction allowed)       */
    SP_PREC_MIXED = 1,      /* FP32 factorisation / Krylov, FP64 residual + update   */
    SP_PREC_FP64_EXACT = 2  /* plain FP64 in the reference's exact operation order,
                               no FMA contraction: bit-identical to the reference on
                               circuits without exp/log device models               */
};

typedef struct sp_ctx sp_ctx;

/* Context lifecycle.  `device` is a CUDA ordinal. */
int sp_ctx_create(int device, sp_ctx** out);
int sp_ctx_destroy(sp_ctx* ctx);
/* Text of the last error on this context ("" if none).  Never NULL. */
const char* sp_ctx_last_error(const sp_ctx* ctx);
/* Library version string, e.g. "spicier-gb300 0.1.0 sm_103a". */
const char* sp_version(void);

/* ---------------------------------------------------------------------- */
/* BatchedLuSolver (solver.rs:107-135)                                    */
/* ---------------------------------------------------------------------- */

/* BatchedLuSolver::backend_type — always SP_BACKEND_GB300. */
int sp_backend_type(void);
/* BatchedLuSolver::should_use_gpu — 1/0. */
int sp_should_use_gpu(const sp_ctx* ctx, size_t matrix_size, size_t batch_size);
/* BatchedLuSolver::config. */
int sp_get_config(const sp_ctx* ctx, sp_batch_config* out);
int sp_set_config(sp_ctx* ctx, const sp_batch_config* cfg);

/* BatchedLuSolver::solve_batch (solver.rs:119-125).
 * matrices: batch*n*n column-major FP64; rhs: batch*n.  On return
 * solutions[batch*n] holds x; singular systems get an all-zero solution and
 * their index in singular_indices (capacity batch), count in *num_singular.
 * Singularity is not an error (CpuBatchedSolver semantics, solver.rs:367-377).
 * Errors: INVALID_DIMENSION (n == 0 with batch > 0), BATCH_TOO_LARGE. */
int sp_solve_batch(sp_ctx* ctx, const double* matrices, const double* rhs,
                   size_t n, size_t batch, double* solutions,
                   uint64_t* singular_indices, uint64_t* num_singular);

/* Same, on device buffers.  singular_flags[batch] receives 1 for a singular
 * system, else 0.  precision: SP_PREC_FP64 (partial-pivot LU in FP64) or
 * SP_PREC_MIXED (FP32 partial-pivot LU + FP64 iterative refinement,
 * refine_steps sweeps; falls back to an FP64 factorisation for a system whose
 * refinement does not reach FP64 accuracy). */
int sp_solve_batch_device(sp_ctx* ctx, const double* d_matrices, const double* d_rhs,
                          size_t n, size_t batch, double* d_solutions,
                          uint8_t* d_singular_flags, int precision, int refine_steps,
                          void* stream);

/* ---------------------------------------------------------------------- */
/* Circuits                                                               */
/* ---------------------------------------------------------------------- */

/* Element kinds: the device set of the Newton path.
 * Field slots (indices into the per-sample parameter vector) per kind:
 *   R:    f[0] resistance (ohm)                          passive.rs:53-59
 *   C:    f[0] capacitance (F); open at DC                passive.rs:232-240
 *   L:    f[0] inductance (H); 0 V source at DC           passive.rs:318-325
 *   V:    f[0] DC voltage                                 sources.rs:96-101
 *   I:    f[0] DC current (flows pos -> neg inside)       sources.rs:230-236
 *   D:    f[0] IS, f[1] N                                 diode.rs:11-38
 *   NMOS/PMOS: f[0] VTO, f[1] KP, f[2] LAMBDA, f[3] W, f[4] L, f[5] NF
 *                                                          mosfet/level1.rs:23-71
 *   NPN/PNP: f[0] IS, f[1] BF, f[2] BR, f[3] NF, f[4] NR, f[5] VAF (<=0: inf)
 *                                                          bjt.rs:23-76
 *   BSIM3N/BSIM3P: f[0] = first of SP_B3_CARD consecutive slots holding the
 *         model card and instance sizes in sp_bsim3_card order
 *                                                          mosfet/bsim3/params.rs
 * node[] holds MNA node indices (0-based, ground = -1):
 *   two-terminal: node[0] = pos/anode, node[1] = neg/cathode
 *   MOSFET: node[0] = drain, node[1] = gate, node[2] = source
 *   BJT:    node[0] = collector, node[1] = base, node[2] = emitter
 *   BSIM3:  node[0] = drain, node[1] = gate, node[2] = source, node[3] = bulk
 *   node[3] is -1 for every other kind.
 * branch: index of the element's current variable (V and L only), else -1;
 *   its MNA row is num_nodes + branch.
 * wave: index into sp_circuit.pulses for a time-varying V/I, else -1. */
enum sp_element_kind {
    SP_EL_R = 1,
    SP_EL_C = 2,
    SP_EL_L = 3,
    SP_EL_V = 4,
    SP_EL_I = 5,
    SP_EL_D = 6,
    SP_EL_NMOS = 7,
    SP_EL_PMOS = 8,
    SP_EL_NPN = 9,
    SP_EL_PNP = 10,
    SP_EL_BSIM3N = 11, /* BSIM3v3.3 DC model (LEVEL=49 / 8), mosfet/bsim3/evaluate.rs */
    SP_EL_BSIM3P = 12
};

/* Parameter slots of a BSIM3 element, relative to its field[0]: the model
 * parameters the DC evaluation reads (Bsim3Params, mosfet/bsim3/params.rs:13-143)
 * with the instance sizes W, L, NF, then those of the small-signal capacitances
 * (AS, AD, PS, PD: 0 = estimated from Weff).  TNOM in kelvin.  Defaults:
 * Bsim3Params::nmos_default / pmos_default (params.rs:160-310). */
enum sp_bsim3_card {
    SP_B3_TOX = 0, SP_B3_LINT, SP_B3_WINT,
    SP_B3_VTH0, SP_B3_K1, SP_B3_K2, SP_B3_DVT0, SP_B3_DVT1, SP_B3_DVT2, SP_B3_NFACTOR,
    SP_B3_K3, SP_B3_K3B, SP_B3_W0, SP_B3_DVT0W, SP_B3_DVT1W, SP_B3_DVT2W,
    SP_B3_U0, SP_B3_UA, SP_B3_UB, SP_B3_UC, SP_B3_VSAT,
    SP_B3_PCLM, SP_B3_PDIBLC1, SP_B3_PDIBLC2, SP_B3_DROUT,
    SP_B3_ETA0, SP_B3_ETAB, SP_B3_DSUB, SP_B3_PDIBLCB, SP_B3_PVAG,
    SP_B3_NCH, SP_B3_TNOM, SP_B3_KT2,
    SP_B3_W, SP_B3_L, SP_B3_NF,
    /* capacitances of the small-signal model (evaluate_capacitances, evaluate.rs:82-158) */
    SP_B3_CGSO, SP_B3_CGDO, SP_B3_CGBO, SP_B3_CJ, SP_B3_CJSW, SP_B3_CJSWG,
    SP_B3_MJ, SP_B3_MJSW, SP_B3_MJSWG, SP_B3_PB, SP_B3_PBSW, SP_B3_PBSWG,
    SP_B3_AS, SP_B3_AD, SP_B3_PS, SP_B3_PD,
    SP_B3_CARD /* number of slots */
};

#define SP_MAX_FIELDS 6

typedef struct sp_element {
    int32_t kind;
    int32_t node[4];
    int32_t branch;
    int32_t wave;
    int32_t field[SP_MAX_FIELDS];
} sp_element;

/* How one per-sample parameter is produced (sweep index s, seed):
 *   FIXED:       a
 *   GAUSS:       gaussian_scaled(seed, s, rng_index, a, b) (rng.rs:148-150),
 *                b is the absolute sigma
 *   UNIFORM:     a + uniform(seed, s, rng_index) * (b - a)
 *   LOGUNIFORM:  a * exp(uniform(seed, s, rng_index) * log(b / a))
 *   TABLE:       column `rng_index` of a caller-supplied [samples][table_cols]
 *                table (host generators: LCG Monte Carlo, corners, linear). */
enum sp_draw_kind {
    SP_DRAW_FIXED = 0,
    SP_DRAW_GAUSS = 1,
    SP_DRAW_UNIFORM = 2,
    SP_DRAW_LOGUNIFORM = 3,
    SP_DRAW_TABLE = 4
};

typedef struct sp_param {
    int32_t kind;
    uint32_t rng_index;
    double a;
    double b;
} sp_param;

/* PULSE(v1 v2 td tr tf pw per), waveforms.rs:159-182. */
typedef struct sp_pulse {
    double v1, v2, td, tr, tf, pw, per;
} sp_pulse;

typedef struct sp_circuit {
    int32_t num_nodes;     /* excluding ground                          */
    int32_t num_branches;  /* current variables: V sources + inductors  */
    int32_t num_elements;
    int32_t num_params;
    int32_t num_pulses;
    int32_t reserved;
    const sp_element* elements;
    const sp_param* params;
    const sp_pulse* pulses;
    /* Optional initial guess [num_nodes + num_branches] used when no per-sample
     * warm start is given (a .nodeset); NULL means zero, the reference's
     * default (newton.rs:80-83). */
    const double* nodeset;
} sp_circuit;

/* Batched BSIM3 DC evaluation (Bsim3Mosfet::evaluate, mosfet/bsim3/evaluate.rs:171-265,
 * with Bsim3Derived::from_params at TNOM, derived.rs:81-196): device i has the
 * card d_card[i][SP_B3_CARD] (sp_bsim3_card order) and the bias
 * d_bias[i][3] = (vgs, vds, vbs); d_out[i][6] receives (ids, gds, gm, gmbs, vth,
 * vdsat) and d_region[i] (optional) 0 subthreshold, 1 linear, 2 saturation.
 * pmos != 0 selects the P-channel sign convention.  The same device function
 * stamps BSIM3 elements in the Newton kernels. */
int sp_bsim3_eval_device(sp_ctx* ctx, int pmos, const double* d_card, const double* d_bias, uint64_t count,
                         double* d_out, uint8_t* d_region, void* stream);

/* Histogram of column `col` of values[rows][ld] (Histogram::new,
 * statistics.rs:243-268): num_bins bins of width (max - min) / num_bins,
 * bin = clamp(floor((v - min) / width), 0, num_bins - 1) (NaN -> bin 0, as
 * Rust's saturating float-to-int cast); rows whose status is not converged
 * are skipped when d_status is given.  d_bins[num_bins] receives the counts
 * (overwritten). */
int sp_histogram_device(sp_ctx* ctx, const double* d_values, uint64_t rows, uint32_t ld,
                        uint32_t col, const uint8_t* d_status, double min, double max,
                        uint32_t num_bins, uint64_t* d_bins, void* stream);

/* Yield (YieldSpec / YieldAnalysis, statistics.rs:331-428): d_pass[k] = rows
 * whose column specs[k].col lies in [lower, upper] (inclusive), d_pass[num_specs]
 * = rows passing every spec; with d_status given, rows that did not converge
 * pass nothing.  Yield = pass / rows. */
typedef struct sp_yield_spec {
    uint32_t col;
    uint32_t reserved;
    double lower, upper;
} sp_yield_spec;
int sp_yield_device(sp_ctx* ctx, const double* d_values, uint64_t rows, uint32_t ld,
                    const uint8_t* d_status, const sp_yield_spec* specs, uint32_t num_specs,
                    uint64_t* d_pass, void* stream);

/* ---------------------------------------------------------------------- */
/* Batched nonlinear transient of RC-diode ladders (no counterpart in the  */
/* reference, whose transient solvers are linear): every instance is a     */
/* ladder of N sections (R in series, C and a Shockley diode to ground)    */
/* driven by a PULSE source, integrated with the reference's TR-BDF2 step  */
/* (companion.rs:41-150, solver.rs:186-251) under the reference's adaptive */
/* step controller (solver.rs:494-676), each stage solved by Newton with   */
/* the reference's convergence test (newton.rs:134-159).                   */
/* ---------------------------------------------------------------------- */
typedef struct sp_ladder_config {
    double tstop, h_init, h_min, h_max;  /* AdaptiveTransientParams (types.rs)   */
    double lte_reltol, lte_abstol;       /* step acceptance tolerance            */
    double v_reltol, v_abstol, i_abstol; /* Newton convergence per stage         */
    double r_lo, r_hi, c_lo, c_hi;       /* log-uniform section R and C ranges   */
    double diode_is, diode_n;            /* Shockley diode of every section      */
    sp_pulse pulse;                      /* source waveform                      */
    int32_t min_sections, max_sections;  /* N = min + floor((max-min+1) u)       */
    int32_t max_iterations;              /* Newton iterations per stage          */
    int32_t max_steps;                   /* accepted + rejected steps per instance */
    int32_t precision;                   /* SP_PREC_*                            */
    int32_t num_probe;                   /* probe samples of v(N) over [0, tstop] */
} sp_ladder_config;

/* Defaults: 4,096-instance workload values (tstop 100 ns, h_init 1 ns,
 * h_min 1 fs, h_max tstop/100, reltol 1e-3, abstol 1e-6, SPICE Newton
 * tolerances, R 100 ohm-10 kohm, C 1-100 pF, IS 1e-14, N 1, PULSE 0->1.8 V
 * with tr = tf = 1 ns, pw 10 ns, per 20 ns, td 0; N in 8..512; 50 Newton
 * iterations; 200,000 steps; FP64; 101 probe samples). */
void sp_ladder_config_default(sp_ladder_config* cfg);

/* Transients of ladder instances first_index .. first_index + count - 1
 * (instance i draws its sections from the hash RNG with sweep index i):
 * x_final[count][max_sections + 2] holds [v_in, v_1..v_N, I_src, 0...] at
 * tstop, n[i] = N + 2, accepted/rejected steps, Newton iterations summed
 * over stages, status (SP_ST_*), probe[count][num_probe] = v_N at
 * j tstop / (num_probe - 1) by linear interpolation between accepted steps. */
int sp_ladder_transient_device(sp_ctx* ctx, const sp_ladder_config* cfg, uint64_t seed,
                               uint64_t first_index, uint64_t count, double* d_x_final,
                               int32_t* d_n, int32_t* d_accepted, int32_t* d_rejected,
                               int32_t* d_iters, uint8_t* d_status, double* d_probe, void* stream);
/* sp_ladder_transient_device that also records the size of every accepted
 * step: d_steps[count][max_steps_recorded] receives instance i's first
 * max_steps_recorded accepted step sizes in order (d_accepted[i] says how
 * many were taken); their prefix sums are the accepted time points, the
 * `time` of each TimePoint in the reference's TransientResult
 * (crates/spicier-solver/src/transient/result.rs:7-16).  Replaying them through
 * the same step arithmetic reproduces the run along its own step sequence. */
int sp_ladder_transient_steps_device(sp_ctx* ctx, const sp_ladder_config* cfg, uint64_t seed,
                                     uint64_t first_index, uint64_t count, double* d_x_final,
                                     int32_t* d_n, int32_t* d_accepted, int32_t* d_rejected,
                                     int32_t* d_iters, uint8_t* d_status, double* d_probe,
                                     double* d_steps, int32_t max_steps_recorded, void* stream);
/* Same on host buffers (copies out; synchronises). */
int sp_ladder_transient(sp_ctx* ctx, const sp_ladder_config* cfg, uint64_t seed, uint64_t first_index,
                        uint64_t count, double* x_final, int32_t* n, int32_t* accepted,
                        int32_t* rejected, int32_t* iters, uint8_t* status, double* probe);

/* ---------------------------------------------------------------------- */
/* Corner sweep of a resistive power-grid mesh with MOSFET current sinks,  */
/* each Newton linear solve by restarted GMRES with Jacobi (right)         */
/* preconditioning (gmres/real.rs:218-397, preconditioner.rs:43-101).      */
/* Instance i: layout i / 4 (edge resistances, sink nodes and gate drives   */
/* from the hash RNG with sweep index i / 4), corner i % 4 (bit 0: all     */
/* resistances x r_scale_hi else x r_scale_lo; bit 1: all VTO + vto_shift  */
/* else - vto_shift).  Unknowns: rows x cols node voltages + the VDD       */
/* branch current; VDD drives corner (0,0), the three other corners are    */
/* tied to it by straps of conductance strap_g; every sink is a Level-1    */
/* NMOS from its node to ground with an ideal gate drive VGS.              */
/* ---------------------------------------------------------------------- */
typedef struct sp_grid_config {
    int32_t rows, cols, num_sinks;
    int32_t max_newton;          /* Newton iterations                      */
    int32_t restart;             /* GMRES(m)                               */
    int32_t max_krylov;          /* GMRES iterations per linear solve      */
    int32_t precision;           /* SP_PREC_FP64 or SP_PREC_MIXED          */
    int32_t reserved;
    double r_lo, r_hi;           /* log-uniform branch resistance          */
    double r_scale_lo, r_scale_hi, vto_shift;
    double vdd, strap_g;
    double vgs_lo, vgs_hi;       /* uniform gate drive                     */
    double vto, kp, lambda, w, l;
    double v_reltol, v_abstol, i_abstol;  /* Newton convergence            */
    double krylov_tol;           /* relative residual of each linear solve */
    double resid_target;         /* final KCL residual bound (A)           */
} sp_grid_config;

/* Defaults: 64 x 64 mesh, 512 sinks, R 0.5-2 ohm x {0.9, 1.1}, VTO 0.7 V
 * +- 50 mV, KP 110e-6, LAMBDA 0.04, W/L 5u/0.5u, VGS 0.8-1.2 V, VDD 1 V,
 * straps 1e3 S, GMRES(30), 1e-9 relative linear tolerance, 20,000 Krylov
 * iterations per solve, 30 Newton iterations, residual target 1e-9 A. */
void sp_grid_config_default(sp_grid_config* cfg);

/* Instances first_index .. first_index + count - 1: x[count][rows*cols+1] at
 * the last Newton iterate, Newton iterations, Krylov iterations summed over
 * the Newton solves, status (SP_ST_*), and the max |KCL residual| over the
 * node rows at x (A).  The mixed precision keeps iterating until the
 * residual also meets resid_target. */
int sp_grid_solve_device(sp_ctx* ctx, const sp_grid_config* cfg, uint64_t seed, uint64_t first_index,
                         uint64_t count, double* d_x, int32_t* d_newton, int32_t* d_krylov,
                         uint8_t* d_status, double* d_resid, void* stream);
/* Same on host buffers (copies out; synchronises). */
int sp_grid_solve(sp_ctx* ctx, const sp_grid_config* cfg, uint64_t seed, uint64_t first_index,
                  uint64_t count, double* x, int32_t* newton, int32_t* krylov, uint8_t* status,
                  double* resid);

/* ConvergenceCriteria (newton.rs:9-34) + stepping parameters
 * (newton.rs:173-231) + backend choices. */
enum sp_fallback_bits {
    SP_FALLBACK_GMIN = 1,    /* solve_with_gmin_stepping on a miss           */
    SP_FALLBACK_SOURCE = 2   /* solve_with_source_stepping after gmin misses */
};

typedef struct sp_newton_config {
    double v_abstol;            /* 1e-6  */
    double v_reltol;            /* 1e-3  */
    double i_abstol;            /* 1e-12 */
    double gmin;                /* 1e-12 (unused by plain Newton, as in the reference) */
    int32_t max_iterations;     /* 50    */
    int32_t precision;          /* sp_precision */
    int32_t fallback;           /* sp_fallback_bits */
    int32_t refine_steps;       /* linear refinement sweeps per Newton step (mixed) */
    double gmin_initial;        /* 1e-3  */
    double gmin_final;          /* 1e-12 */
    double gmin_reduction;      /* 10    */
    int32_t gmin_max_attempts;  /* 5     */
    int32_t src_max_attempts;   /* 5     */
    double src_initial;         /* 0.1   */
    double src_step;            /* 0.1   */
    double src_min_step;        /* 0.01  */
    int32_t warm_max_iterations; /* cap of the attempt from a warm start before the
                                    cold restart (0: max_iterations) */
    int32_t reserved;
} sp_newton_config;

/* Fill *cfg with the reference defaults (plain FP64, gmin+source fallback). */
void sp_newton_config_default(sp_newton_config* cfg);

/* Per-sample status byte (ConvergenceStatus, convergence.rs:41-50, with
 * flag bits saying which path produced the answer). */
enum sp_sample_status {
    SP_ST_CONVERGED = 0,
    SP_ST_FAILED = 1,      /* iteration caps hit on every path              */
    SP_ST_SINGULAR = 2,    /* a linearised system had a zero pivot           */
    SP_ST_NONFINITE = 3,   /* NaN/Inf appeared in the iterate                */
    SP_ST_MASK = 0x0f,
    SP_ST_FLAG_WARM = 0x10,     /* started from the caller's warm start       */
    SP_ST_FLAG_COLD = 0x20,     /* warm start missed; cold Newton was used    */
    SP_ST_FLAG_GMIN = 0x40,     /* answer came from gmin stepping            */
    SP_ST_FLAG_SOURCE = 0x80    /* answer came from source stepping          */
};

/* StatisticsAccumulator (statistics.rs:113-160): raw moments of one
 * unknown over the converged samples. */
typedef struct sp_moments {
    uint64_t count;
    double sum;
    double sum_sq;
    double min;
    double max;
} sp_moments;

/* A circuit uploaded to the device once and reused across sweeps. */
typedef struct sp_topology sp_topology;
int sp_topology_create(sp_ctx* ctx, const sp_circuit* circuit, sp_topology** out);
int sp_topology_destroy(sp_topology* topo);
/* Number of MNA unknowns (nodes + branches). */
int sp_topology_size(const sp_topology* topo);

/* Topology-specialised Newton kernel for `precision` (SP_PREC_MIXED or
 * SP_PREC_FP64): the element list, the sparsity pattern and a static pivot
 * order (partial pivoting of the Jacobian at the nominal operating point)
 * with its symbolic fill are compiled into straight-line register code with
 * NVRTC (the cached symbolic factorisation of CachedSparseLu,
 * crates/spicier-solver/src/linear.rs:334-410, fixed at compile time).
 * enable != 0 builds it (once) and uses it for later sweeps of that
 * precision; enable == 0 returns to the generic kernels.  SP_PREC_MIXED is
 * specialised automatically on first use unless disabled here.  log (optional)
 * receives the compiler log or the reason for a failure. */
int sp_topology_specialize(sp_ctx* ctx, sp_topology* topo, int precision, int enable,
                           char* log, size_t log_len);

/* The CUDA source of a circuit's specialised kernel, without a device: fills
 * src (capacity src_len, truncated) and, when compile != 0, compiles it with
 * NVRTC for sm_103a (the compiler log goes to src on failure).  *nnz (optional)
 * receives the number of Jacobian slots (structural nonzeros + fill). */
int sp_specialize_source(const sp_circuit* circuit, int precision, int compile, char* src,
                         size_t src_len, int* nnz);

/* Batched DC operating points on device buffers.
 *   Samples are sweep indices first_index .. first_index + num_samples - 1;
 *   draws are keyed by (seed, sweep index, rng_index) so any split of a sweep
 *   gives identical results.
 *   d_table: [num_samples][table_cols] FP64 for SP_DRAW_TABLE parameters
 *            (may be NULL when the circuit has none).
 *   d_x0:    optional [num_samples][n] warm starts.  NULL: start from the
 *            circuit's nodeset, or zero without one (newton.rs:80-83).  With
 *            a warm start, a miss restarts cold from the nodeset (or zero)
 *            before the gmin/source-stepping fallbacks.
 *   d_x:     [num_samples][n] solutions (written for every sample).
 *   d_iters: [num_samples] total Newton iterations over all paths (optional).
 *   d_status:[num_samples] sp_sample_status bytes (optional).
 *   d_resid: [num_samples] max over node rows of |KCL residual| (A) of the
 *            returned x, evaluated in FP64 (optional).
 *   d_params:[num_samples][num_params] the drawn parameters (optional).
 *   d_moments: [n] moments over converged samples (optional). */
int sp_newton_dc_device(sp_ctx* ctx, const sp_topology* topo,
                        const sp_newton_config* cfg, uint64_t seed,
                        uint64_t first_index, uint64_t num_samples,
                        const double* d_table, uint32_t table_cols,
                        const double* d_x0, double* d_x, int32_t* d_iters,
                        uint8_t* d_status, double* d_resid, double* d_params,
                        sp_moments* d_moments, void* stream);

/* Same on host buffers (copies in and out; synchronises). */
int sp_newton_dc(sp_ctx* ctx, const sp_circuit* circuit,
                 const sp_newton_config* cfg, uint64_t seed,
                 uint64_t first_index, uint64_t num_samples,
                 const double* table, uint32_t table_cols,
                 const double* x0, double* x, int32_t* iters,
                 uint8_t* status, double* resid, double* params,
                 sp_moments* moments);

/* sp_newton_dc_device without any device allocation.  No counterpart in the
 * reference.  For callers that cannot let a library call cudaMalloc — a host
 * application whose device memory belongs to its own pool, a process under a
 * hard device-memory cap, a loop that cannot take cudaMalloc's implicit
 * device synchronisation.  No context, no topology: the circuit is copied
 * from host memory into a fixed 16 MiB file-scope device array that also
 * holds the drawn parameters, derived constants and fallback miss list
 * (every GPU that loads the library holds it until exit); sweeps needing more
 * are rejected with SP_ERR_BATCH_TOO_LARGE.  Runs on the current device.  The
 * first call on a device does a one-time set-up (it looks up the array's
 * address with cudaGetSymbolAddress): make it before any stream capture.
 * Every call copies the circuit from pageable host memory, so a call whose
 * stream is capturing returns SP_ERR_INVALID_ARGUMENT and enqueues nothing.
 * The set-up is kept per device ordinal: cudaDeviceReset after the first
 * call is not supported.  All calls on a device share the array, so calls
 * that overlap on the GPU race; order them.  Outputs as for
 * sp_newton_dc_device (no moments); err
 * (optional, err_len bytes) receives a message on failure. */
int sp_newton_dc_static(const sp_circuit* circuit, const sp_newton_config* cfg,
                        uint64_t seed, uint64_t first_index, uint64_t num_samples,
                        const double* d_table, uint32_t table_cols,
                        const double* d_x0, double* d_x, int32_t* d_iters,
                        uint8_t* d_status, double* d_resid, void* stream,
                        char* err, size_t err_len);

/* ---------------------------------------------------------------------- */
/* Batched fixed-step linear transients (solve_transient, solver.rs:41-252): */
/* the DC operating point of each sample (the Newton path, cfg as for       */
/* sp_newton_dc), then num_steps = ceil(tstop / tstep) steps of BE, TRAP or */
/* TR-BDF2 with the reference's companion models (companion.rs).  Circuits  */
/* are linear (R, C, L, V, I; V and I may carry a PULSE).  Transient        */
/* unknowns: nodes, then the V-source currents in element order.            */
/* ---------------------------------------------------------------------- */
enum sp_transient_method { SP_TRAN_BE = 0, SP_TRAN_TRAP = 1, SP_TRAN_TRBDF2 = 2 };
typedef struct sp_transient_config {
    double tstep, tstop;
    int32_t method;     /* sp_transient_method                                   */
    int32_t probe;      /* transient unknown recorded at every step, -1: none    */
    int32_t precision;  /* SP_PREC_FP64 or SP_PREC_FP64_EXACT                    */
    int32_t reserved;
} sp_transient_config;

/* x[count][nt] = state at the last step; probe[count][num_steps + 1] (when
 * probe >= 0); status: the DC status, or SP_ST_SINGULAR when a step's solve
 * hit a zero pivot (probe entries after it are NaN). */
int sp_transient_device(sp_ctx* ctx, const sp_topology* topo, const sp_newton_config* dc_cfg,
                        const sp_transient_config* tc, uint64_t seed, uint64_t first_index,
                        uint64_t count, const double* d_table, uint32_t table_cols, double* d_x,
                        double* d_probe, uint8_t* d_status, void* stream);
int sp_transient(sp_ctx* ctx, const sp_circuit* circuit, const sp_newton_config* dc_cfg,
                 const sp_transient_config* tc, uint64_t seed, uint64_t first_index, uint64_t count,
                 const double* table, uint32_t table_cols, double* x, double* probe, uint8_t* status);

/* ---------------------------------------------------------------------- */
/* Batched AC small-signal sweeps (solve_ac, ac.rs:357-400, with the netlist */
/* AC stamper of crates/spicier-cli/src/stampers.rs): per sample the DC      */
/* operating point (the Newton path, cfg as for sp_newton_dc), the devices'  */
/* small-signal conductances there (ac_info_at), and at every frequency the */
/* complex MNA solve with the reference's dense LU.  Unknowns: nodes, then  */
/* the branch currents (V sources and inductors) as in the DC path.         */
/* ---------------------------------------------------------------------- */
enum sp_ac_sweep_type { SP_AC_LIN = 0, SP_AC_DEC = 1, SP_AC_OCT = 2 };
typedef struct sp_ac_config {
    double fstart, fstop;
    int32_t num_points;  /* total (linear) or per decade / octave              */
    int32_t sweep;       /* sp_ac_sweep_type                                   */
    int32_t source;      /* -1: every V source at AC magnitude 1 (ac_info's   */
                         /* default); else the element index of the stimulus */
    int32_t num_probe;   /* 1..8 unknowns recorded                             */
    int32_t probe[8];
    int32_t precision;   /* SP_PREC_FP64: the reference's FP64 LU order;       */
                         /* SP_PREC_MIXED: FP32 complex LU + FP64 refinement  */
    int32_t refine;      /* mixed: residual refinement steps (0 -> 3)          */
} sp_ac_config;

/* The frequency grid (generate_frequencies, ac.rs:258-287): writes up to cap
 * values to freqs (may be NULL) and returns the number of frequencies. */
int sp_ac_frequencies(const sp_ac_config* cfg, double* freqs, int cap);
/* probe[count][nf][num_probe] complex values as (re, im) double pairs;
 * status: the DC status, or SP_ST_SINGULAR when a frequency's matrix was
 * singular (that frequency's probes NaN).  Samples whose DC point did not
 * converge get NaN probes. */
int sp_ac_sweep_device(sp_ctx* ctx, const sp_topology* topo, const sp_newton_config* dc_cfg,
                       const sp_ac_config* ac, uint64_t seed, uint64_t first_index, uint64_t count,
                       const double* d_table, uint32_t table_cols, double* d_probe, uint8_t* d_status,
                       void* stream);
int sp_ac_sweep(sp_ctx* ctx, const sp_circuit* circuit, const sp_newton_config* dc_cfg, const sp_ac_config* ac,
                uint64_t seed, uint64_t first_index, uint64_t count, const double* table, uint32_t table_cols,
                double* probe, uint8_t* status);

/* ---------------------------------------------------------------------- */
/* Learned Newton warm start (no counterpart in the reference).            */
/* A BF16 MLP n_in -> n_layers x n_hidden (GELU) -> n_out, trained and run */
/* on the tensor cores with FP32 accumulation; FP32 master weights + Adam. */
/* ---------------------------------------------------------------------- */
typedef struct sp_mlp sp_mlp;
typedef struct sp_mlp_desc {
    int32_t n_in;       /* <= 64 */
    int32_t n_hidden;   /* multiple of 32, <= 1024 */
    int32_t n_layers;   /* hidden layers, 1..8 */
    int32_t n_out;      /* <= 64 */
    uint64_t init_seed; /* He-uniform initialisation from the hash RNG */
} sp_mlp_desc;

int sp_mlp_create(sp_ctx* ctx, const sp_mlp_desc* desc, sp_mlp** out);
int sp_mlp_destroy(sp_mlp* mlp);
/* Flat FP32 parameters: per layer Wt[out_pad][in_pad] then b[out_pad], where
 * in/out of the first/last layer are padded to multiples of 32. */
int sp_mlp_num_params(const sp_mlp* mlp);
int sp_mlp_get_params(sp_mlp* mlp, float* host_params);
int sp_mlp_set_params(sp_mlp* mlp, const float* host_params);
/* Warm-start wiring: input j is circuit parameter slot in_slots[j],
 * normalised as (p - in_mean[j]) / in_scale[j]; output k is MNA unknown k,
 * x0[k] = out_mean[k] + out_scale[k] * y[k] (n_out must equal the MNA size). */
int sp_mlp_set_io(sp_mlp* mlp, const int32_t* in_slots, const float* in_mean,
                  const float* in_scale, const float* out_mean, const float* out_scale);
/* FP64 linear term of the warm start, lin[n_out][n_in] (NULL removes it):
 * x0[k] = out_mean[k] + out_scale[k] * y[k] + sum_j lin[k][j] * (p_j - in_mean[j]).
 * The network then only has to learn what is not linear in the inputs. */
int sp_mlp_set_linear(sp_mlp* mlp, const double* lin);
/* Inference kernel of the warm start.  AUTO picks the tcgen05 kernel (TMEM
 * accumulators; weights resident in shared memory for hidden 64 or 128,
 * streamed from L2 through shared-memory slots for hidden 256) when the
 * shape allows it (n_in <= 32, n_out <= 32, hidden 64, 128 or 256, 1..4
 * hidden layers), else the fused mma.sync kernel (hidden <= 256), else the
 * layer-by-layer GEMMs. */
enum sp_mlp_kernel {
    SP_MLP_KERNEL_AUTO = 0,
    SP_MLP_KERNEL_TCGEN05 = 1,
    SP_MLP_KERNEL_MMA_SYNC = 2,
    SP_MLP_KERNEL_LAYERED = 3,
    /* the linear term alone (sp_mlp_set_linear and the I/O mapping, no
     * network): x0[k] = out_mean[k] + sum_j lin[k][j] (p_j - in_mean[j]) in
     * FP32, evaluated by the learned sweep's draw kernel from the parameters
     * it has just drawn, so no inference kernel runs */
    SP_MLP_KERNEL_LINEAR = 4
};
int sp_mlp_set_inference_kernel(sp_mlp* mlp, int kind);
/* Kernel of the training GEMMs (forward, data gradient, weight gradient):
 * AUTO and TCGEN05 run them on the tensor cores (tcgen05.mma, FP32
 * accumulators in TMEM; TCGEN05 requires a hidden width that is a multiple of
 * 16), MMA_SYNC on the legacy mma.sync kernel.  LAYERED is not a training
 * kernel. */
int sp_mlp_set_training_kernel(sp_mlp* mlp, int kind);
/* Waits for the device, then *fault = 1 if a tcgen05 training GEMM gave up a
 * bounded wait (its results are invalid), | 2 if the tcgen05 warm start did
 * (those samples started cold); 0 otherwise.  The flags are sticky. */
int sp_mlp_fault(sp_mlp* mlp, int* fault);
/* The warm start alone: x0[rows][n_out] (FP64) from per-sample parameters in
 * structure-of-arrays layout (parameter slot s of sample i at
 * d_params_soa[s * stride + i]), with the I/O mapping and linear term above. */
int sp_mlp_warm_start_device(sp_mlp* mlp, const double* d_params_soa, uint64_t stride,
                             uint64_t rows, double* d_x0, void* stream);
/* y[rows][n_out] = net(x[rows][n_in]) on normalised FP32 data. */
int sp_mlp_forward_device(sp_mlp* mlp, const float* d_x, uint64_t rows, float* d_y,
                          void* stream);
/* Mean-squared-error gradients of one batch (rows a multiple of 64) into
 * d_grads[num_params] (flat layout above); *d_loss = the batch loss. */
int sp_mlp_gradients_device(sp_mlp* mlp, const float* d_x, const float* d_t, uint64_t rows,
                            float* d_grads, float* d_loss, void* stream);
/* Adam training over rows/batch contiguous batches per epoch, cosine learning
 * rate decay from lr to lr/100; d_epoch_loss[e] (optional) = sum over the
 * epoch's batches of the batch loss. */
int sp_mlp_train_device(sp_mlp* mlp, const float* d_x, const float* d_t, uint64_t rows,
                        int batch, int epochs, float lr, float* d_epoch_loss, void* stream);

/* Batched DC operating points started from the network's prediction:
 * parameters are drawn once, the network maps them to an FP64 warm start, and
 * Newton runs from there; a miss restarts from the circuit's nodeset and then
 * the gmin/source-stepping chain (cfg.fallback).  Outputs as for
 * sp_newton_dc_device. */
int sp_newton_dc_learned_device(sp_ctx* ctx, const sp_topology* topo, sp_mlp* mlp,
                                const sp_newton_config* cfg, uint64_t seed,
                                uint64_t first_index, uint64_t num_samples,
                                const double* d_table, uint32_t table_cols, double* d_x,
                                int32_t* d_iters, uint8_t* d_status, double* d_resid,
                                sp_moments* d_moments, void* stream);

/* Same on host buffers (copies in and out; synchronises). */
int sp_newton_dc_learned(sp_ctx* ctx, const sp_circuit* circuit, sp_mlp* mlp,
                         const sp_newton_config* cfg, uint64_t seed, uint64_t first_index,
                         uint64_t count, const double* table, uint32_t table_cols, double* x,
                         int32_t* iters, uint8_t* status, double* resid, sp_moments* moments);

/* Draw the per-sample parameter vectors only ([num_samples][num_params]). */
int sp_draw_params_device(sp_ctx* ctx, const sp_topology* topo, uint64_t seed,
                          uint64_t first_index, uint64_t num_samples,
                          const double* d_table, uint32_t table_cols,
                          double* d_params, void* stream);

/* The same draws on the host, with the C library's ln, cos and exp, in the
 * reference's operation order (generate_gaussian_parameters and
 * gaussian_scaled, rng.rs:120-150 and 208-227): out[num_samples][num_params]
 * for sweep indices first_index ..  The reference's Gaussian draws are its
 * host libm's bits, which are not correctly rounded; the device draws are
 * correctly rounded and agree with glibc in about 99.8 % of draws.  A sweep
 * given this table (each slot read as a table column) runs on the
 * reference's own draws on this host.  threads <= 0: all host threads.
 * Table parameters copy table[i][col] (NaN without a table).  Needs no GPU. */
int sp_draw_params_host(const sp_circuit* circuit, uint64_t seed, uint64_t first_index,
                        uint64_t num_samples, const double* table, uint32_t table_cols,
                        double* out, int threads);

/* Raw hash RNG on device (rng.rs:39-150): out[i] for sweep index
 * first_index + i and parameter param_index.  kind: 0 uniform, 1 gaussian,
 * 2 uniform_f32 (as double), 3 gaussian_f32 (as double). */
int sp_rng_fill_device(sp_ctx* ctx, int kind, uint64_t seed, uint64_t first_index,
                       uint32_t param_index, uint64_t count, double* d_out, void* stream);

/* ---------------------------------------------------------------------- */
/* Kernel timing (tracing).  The reference has only log macros and ad-hoc  */
/* timers (crates/spicier-backend-metal/src/gpu_newton.rs:128); this adds  */
/* CUDA-event timing around every kernel the library launches.             */
/* ---------------------------------------------------------------------- */
typedef struct sp_kernel_time {
    char name[48];
    uint64_t launches;
    double total_ms;
} sp_kernel_time;

/* Start (on != 0) or stop recording events around each launch. */
int sp_profile_enable(sp_ctx* ctx, int on);
/* Synchronise, aggregate the recorded launches by kernel name into out
 * (capacity cap), set *count, and clear the record. */
int sp_profile_read(sp_ctx* ctx, sp_kernel_time* out, int cap, int* count);

/* Moments of column `col` of a [rows][ld] FP64 matrix restricted to rows
 * whose mask byte (optional) has (mask & SP_ST_MASK) == SP_ST_CONVERGED. */
int sp_moments_device(sp_ctx* ctx, const double* d_values, uint64_t rows, uint32_t ld,
                      uint32_t cols, const uint8_t* d_status, sp_moments* d_out,
                      void* stream);

/* ---------------------------------------------------------------------- */
/* Launch settings chosen by an autotuner (no counterpart in the reference, */
/* whose dispatch thresholds are fixed, crates/spicier-solver/src/         */
/* dispatch.rs:85-120).  A setting applies to the sizes of one bucket: key */
/* "<setting>@<bucket>", bucket = sp_tune_bucket(size) (the smallest power */
/* of two >= size, at least 4).  Settings and their size:                  */
/*   lu.cta               1: CTA-per-system batched LU even where one      */
/*                        thread per system fits (n <= 28); size n         */
/*   newton.block.fp64 | .mixed | .exact  threads per block of the generic */
/*                        thread-per-sample Newton kernels; size MNA n     */
/*   spec.bpsm.fp64 | .mixed  resident blocks per SM of the topology-      */
/*                        specialised kernel (at most the occupancy limit) */
/*   ladder.bpsm          resident blocks per SM of the ladder transients  */
/*                        (at most what fits); size max_sections           */
/*   mlp.teams            128-sample tiles in flight per SM of the tcgen05 */
/*                        warm start (resident weights); size hidden width */
/* value <= 0 removes a setting.  Results do not depend on any setting.    */
/* sp_tune_get returns 1 and the value when the key is set, else 0.        */
/* ---------------------------------------------------------------------- */
int sp_tune_set(sp_ctx* ctx, const char* key, int value);
int sp_tune_get(sp_ctx* ctx, const char* key, int* value);
int sp_tune_bucket(long long size);

/* StatisticsAccumulator::merge (statistics.rs:148-155) for n unknowns:
 * acc[i] absorbs other[i] (counts and sums added, min/max combined), as
 * StreamingStatistics::merge (statistics.rs:548-559) does per node.  This is
 * how the moments of chunked sweeps, or of the sample ranges of several
 * processes, combine into the moments of the whole sweep.  The device form
 * runs on `stream`; the host form needs no GPU. */
int sp_moments_merge_device(sp_ctx* ctx, sp_moments* d_acc, const sp_moments* d_other,
                            uint32_t n, void* stream);
int sp_moments_merge(sp_moments* acc, const sp_moments* other, uint32_t n);

#ifdef __cplusplus
}
#endif

#endif /* SPICIER_GB300_H */
