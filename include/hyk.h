/*
 * hyk.h - C ABI of the GB300 batch Taylor integrator (libhyk.so).
 *
 * This library replaces the hot path of heyoka.py's batch-mode integrator
 * (heyoka::taylor_adaptive_batch<double>, driven from
 * heyoka/expose_batch_integrators.cpp) with FP64 CUDA kernels generated per
 * ODE system and compiled with NVRTC for sm_103a.
 *
 * Conventions
 *  - Plain C types only: no C++ exceptions, no torch types.  Every entry point
 *    returns 0 on success or a negative HYK_ERR_* code; the message of the
 *    last failure on the calling thread is returned by hyk_last_error().
 *  - Device arrays are borrowed: the caller allocates them (e.g. as torch
 *    tensors) and keeps them alive until the work on `stream` completes.  The
 *    library allocates device memory only for compiled modules.
 *  - Per-lane arrays use the reference's [var][lane] row-major layout: state
 *    is (n_eq, n_lanes), pars (n_pars, n_lanes), Taylor coefficients
 *    (n_eq, order + 1, n_lanes), grid output (n_grid, n_eq, n_lanes)
 *    (heyoka/expose_batch_integrators.cpp:116-119, :378-382, :481-483).
 *  - `stream` is a cudaStream_t / CUstream passed as void* (NULL = legacy
 *    default stream).  All work is stream-ordered; nothing blocks except
 *    hyk_module_create().
 */
#ifndef HYK_H
#define HYK_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Taylor decomposition (input to module creation and to the oracle) ---- */

/* Elementary operations of the Taylor decomposition.  Mirrors the u-variable
 * vocabulary of the reference's decomposition property
 * (heyoka/expose_batch_integrators.cpp:231). */
enum {
    HYK_OP_ADD = 0,
    HYK_OP_SUB = 1,
    HYK_OP_MUL = 2,
    HYK_OP_DIV = 3,
    HYK_OP_NEG = 4,
    HYK_OP_SQUARE = 5,
    HYK_OP_SQRT = 6,
    HYK_OP_POW = 7, /* exponent: b.num (b.kind == HYK_ARG_NUM) */
    HYK_OP_EXP = 8,
    HYK_OP_LOG = 9,
    HYK_OP_SIN = 10, /* aux = index of the partner cosine u-variable */
    HYK_OP_COS = 11  /* aux = index of the partner sine u-variable */
};

enum { HYK_ARG_NONE = 0, HYK_ARG_U = 1, HYK_ARG_NUM = 2, HYK_ARG_PAR = 3, HYK_ARG_TIME = 4 };

typedef struct hyk_arg {
    int32_t kind; /* HYK_ARG_* */
    int32_t idx;  /* u-variable index (HYK_ARG_U) or parameter index (HYK_ARG_PAR) */
    double num;   /* value (HYK_ARG_NUM) */
} hyk_arg_t;

typedef struct hyk_uop {
    int32_t op;  /* HYK_OP_* */
    int32_t aux; /* sin/cos partner, else -1 */
    hyk_arg_t a;
    hyk_arg_t b; /* kind HYK_ARG_NONE for unary operations */
} hyk_uop_t;

/* u-variables 0..n_eq-1 are the state variables, u-variable n_eq + k is
 * defined by ops[k] (topological order), rhs[i] is the right-hand side of
 * state variable i. */
typedef struct hyk_decomp {
    uint32_t n_eq;
    uint32_t n_ops;
    uint32_t n_pars;
    uint32_t n_ev;              /* number of events (0: none) */
    const hyk_uop_t *ops;
    const hyk_arg_t *rhs;
    const struct hyk_event *ev; /* (n_ev) event functions, or NULL */
} hyk_decomp_t;

/* An event of the batch integrator (heyoka's t_event_batch / nt_event_batch,
 * heyoka/taylor_expose_events.cpp:202-311): the event function g (an
 * argument of the decomposition, normally the u-variable of the event
 * expression, decomposed together with the system) and how its roots act.
 * Every step the Taylor polynomial of g over the step is searched for roots;
 * a terminal event ends the step at its first root (outcome = the event's
 * index among the terminal events), a non-terminal event's roots are
 * recorded (time, direction) for the host to report. */
typedef struct hyk_event {
    hyk_arg_t g;
    int32_t terminal;  /* 1: terminal, 0: non-terminal */
    int32_t direction; /* -1: only roots where g decreases, +1: increases, 0: any */
    double cooldown;   /* terminal: after a trigger the event is ignored for this time; < 0: automatic */
} hyk_event_t;

/* ---- taylor_outcome (values of heyoka/core.cpp:324-329, as printed in
 *      doc/notebooks/Batch mode overview.ipynb) ---- */
#define HYK_OUTCOME_SUCCESS (-4294967297LL)
#define HYK_OUTCOME_STEP_LIMIT (-4294967298LL)
#define HYK_OUTCOME_TIME_LIMIT (-4294967299LL)
#define HYK_OUTCOME_ERR_NF_STATE (-4294967300LL)
#define HYK_OUTCOME_CB_STOP (-4294967301LL)

/* ---- error codes ---- */
#define HYK_OK 0
#define HYK_ERR_INVALID (-1)  /* invalid argument */
#define HYK_ERR_CUDA (-2)     /* CUDA driver / runtime failure */
#define HYK_ERR_NVRTC (-3)    /* kernel compilation failure */
#define HYK_ERR_UNSUPPORTED (-4)
#define HYK_ERR_TIMEOUT (-5)  /* a bounded device wait gave up */

/* ---- GPU module: one decomposition compiled at one Taylor order ---- */

typedef struct hyk_module hyk_module;

typedef struct hyk_config {
    uint32_t block_lanes;  /* threads per CTA; 0 = autotune */
    uint32_t persist_ctas; /* CTAs per SM of the persistent kernel; 0 = occupancy-derived */
    uint32_t flags;        /* HYK_CFG_* */
    uint32_t team_size;    /* threads per trajectory: 0 = chosen per system, 1 = one thread per
                              trajectory (lane form), 2..32 (power of two) = team form */
} hyk_config_t;

#define HYK_CFG_PIN_ARITH 1u /* oracle "pin" arithmetic: no FMA, divide by n (slower; for cross-checks) */
#define HYK_CFG_ADJOINT 2u   /* also generate the adjoint (reverse-mode) kernel for hyk_adjoint() */
#define HYK_CFG_HIGH_ACCURACY 4u /* state update by compensated summation (the reference's high_accuracy) */
#define HYK_CFG_FLOAT32 16u      /* single precision: every real array of the lanes and of hyk_prop_t is float
                                    (heyoka's float32 batch integrator); not with pin arithmetic, the
                                    adjoint or events */
#define HYK_CFG_GLOBAL_JETS 8u   /* one thread per trajectory with the Taylor coefficients in global memory
                                    (chosen automatically for systems that leave fewer than two warps
                                    per SM in shared memory) */
#define HYK_CFG_NO_COLD_ROWS 32u /* keep every state variable's coefficients in shared memory.
                                    By default, when that lets more lanes (trajectories) share an SM,
                                    the lane form keeps orders 1..p of the variables that no recurrence
                                    reads at a later order in a module-owned global buffer, and the team
                                    form, when no recurrence reads any state variable at a later order,
                                    keeps two shared slots per state variable and all orders in that
                                    buffer (the module's calls must then be ordered on one stream, as
                                    with HYK_CFG_GLOBAL_JETS) */
#define HYK_CFG_DEBUG 64u        /* debug build of the module's kernels (slower): lane indices taken from a
                                    lane list or a serving ring are checked against n_lanes, and a Taylor
                                    coefficient of a state variable that is not finite is recorded with
                                    its lane, variable, order and iteration; nothing traps, every finding
                                    goes to the module's debug record (hyk_module_debug) */

typedef struct hyk_module_info {
    uint32_t n_eq, n_pars, order, n_u;
    uint32_t block_lanes;        /* threads per CTA used by the kernels */
    uint32_t smem_per_lane;      /* bytes of shared-memory jet storage per lane; 0 when the system is
                                    too large for shared memory and its coefficients live in a
                                    module-owned global buffer */
    uint32_t regs_per_thread;    /* from the compiled kernel */
    uint32_t ctas_per_sm;        /* resident CTAs per SM of the propagate kernel */
    uint32_t n_sm;
    uint32_t reserved;
    double flops_per_step;       /* algorithmic FP64 flops of one Taylor step of one lane */
    double compile_seconds;
    uint32_t team_size;          /* threads per trajectory (1 = lane form) */
    uint32_t reserved2;
} hyk_module_info_t;

/* Decompose-compile-load.  Replaces the construction of
 * heyoka::taylor_adaptive_batch<double> (decomposition + order selection + JIT,
 * heyoka/expose_batch_integrators.cpp:166-208).  `order` >= 2.  `device` is a
 * CUDA device ordinal.  Compiled kernels are cached per process by
 * (decomposition, order, config). */
int hyk_module_create(const hyk_decomp_t *d, uint32_t order, const hyk_config_t *cfg, int device,
                      hyk_module **out);
int hyk_module_destroy(hyk_module *m);
int hyk_module_get_info(const hyk_module *m, hyk_module_info_t *info);
/* Debug record of a module created with HYK_CFG_DEBUG (HYK_ERR_INVALID for
 * any other module).  out[0]: the OR of every HYK_DBG_* code seen since the
 * last clear; out[1]: how many findings; out[2]: the code of the first
 * finding and out[3..6] its details:
 *   HYK_DBG_LANE_RANGE: the lane index, n_lanes, the list position, 0;
 *   HYK_DBG_NONFINITE_JET: lane, state variable, order, iteration;
 *   HYK_DBG_CAPACITY: lane, iteration, 0, 0.
 * Reads device memory synchronously: the caller synchronises the streams
 * the module's launches ran on first.  `clear` non-zero zeroes the record
 * afterwards. */
#define HYK_DBG_LANE_RANGE 1u    /* a lane list or ring entry >= n_lanes (skipped) */
#define HYK_DBG_NONFINITE_JET 2u /* a state variable's Taylor coefficient was not finite */
#define HYK_DBG_CAPACITY 4u      /* a lane stopped on tc/ck/event capacity */
int hyk_module_debug(hyk_module *m, uint64_t out[8], int clear);

/* The generated CUDA source of the module (valid until hyk_module_destroy). */
const char *hyk_module_source(const hyk_module *m);

/* Lane data, device pointers, row stride `ld` (>= n_lanes) for 2-D arrays.
 * A module created with HYK_CFG_FLOAT32 (heyoka's taylor_adaptive_batch<float>)
 * reads and writes float arrays through every real pointer of hyk_lanes_t,
 * hyk_step and hyk_prop_t: the caller passes float buffers cast to double *. */
typedef struct hyk_lanes {
    uint64_t n_lanes;
    uint64_t ld;
    double *state;         /* (n_eq, ld) in/out */
    const double *pars;    /* (n_pars, ld) or NULL when n_pars == 0 */
    double *time_hi;       /* (n_lanes) double-length time, in/out */
    double *time_lo;       /* (n_lanes) */
} hyk_lanes_t;

/* One Taylor step on every lane.  Replaces taylor_adaptive_batch::step /
 * step(max_delta_t) / step_backward (heyoka/expose_batch_integrators.cpp:233-241,
 * reference method bodies in the heyoka C++ library).
 *   max_delta_t: (n_lanes) signed step limits, or NULL for +inf (forward step);
 *                pass `backward` = 1 with NULL for step_backward (-inf).
 *   outcome:     (n_lanes) int64 taylor_outcome per lane (out)
 *   h:           (n_lanes) step taken per lane (out)
 *   tc:          (n_eq, order+1, n_lanes) Taylor coefficients of the step, or NULL
 *   ev:          event buffers (the ev_* fields of a hyk_prop_t; the other
 *                fields are ignored), or NULL; needed when the module has
 *                events.  A terminal event ends the step at its root: the
 *                outcome is the event's index and ev_sign the root's direction. */
struct hyk_prop;
int hyk_step(hyk_module *m, const hyk_lanes_t *lanes, const double *max_delta_t, int backward,
             int64_t *outcome, double *h, double *tc, const struct hyk_prop *ev, void *stream);

/* Propagation of every lane to its own final time.  Replaces
 * taylor_adaptive_batch::propagate_until / propagate_for / propagate_grid
 * (heyoka/expose_batch_integrators.cpp:243-392).  Each lane follows the
 * reference's per-lane rules (double-length remaining time, step clamped to
 * the remaining time and to max_delta_t, zero steps not counted, per-lane
 * outcome / min |h| / max |h| / step count).
 *
 * The per-lane bookkeeping arrays are caller-owned device memory and are both
 * input and output, so a propagation can be resumed (hyk_prop_init fills them
 * from the targets; hyk_propagate advances them). */
typedef struct hyk_prop {
    /* targets and limits */
    const double *tf_hi;       /* (n_lanes) final time, double-length */
    const double *tf_lo;       /* (n_lanes) */
    const double *max_delta_t; /* (n_lanes) >= 0, or NULL for +inf */
    uint64_t max_steps;        /* 0 = unlimited; iterations per lane */
    /* optional dense output over a grid: grid (n_grid, ld), out (n_grid, n_eq, ld) */
    const double *grid;
    uint64_t n_grid;
    double *grid_out;
    /* optional per-step Taylor-coefficient capture (continuous output):
     * tc_out (tc_capacity, n_eq, order+1, ld), tc_t_hi/lo (tc_capacity, ld) =
     * time at the END of each captured step */
    double *tc_out;
    double *tc_t_hi;
    double *tc_t_lo;
    uint64_t tc_capacity;
    /* per-lane bookkeeping, in/out */
    double *rem_hi;      /* remaining time (double-length) */
    double *rem_lo;
    int64_t *outcome;    /* last outcome */
    double *min_h;
    double *max_h;
    uint64_t *n_steps;   /* accepted non-zero steps */
    uint64_t *n_iter;    /* iterations (steps attempted, incl. zero) */
    uint64_t *grid_idx;  /* next grid row to write */
    double *last_h;      /* h of the last iteration */
    double *last_tc;     /* (n_eq, order+1, ld) Taylor coefficients of the last step, or NULL */
    uint32_t *status;    /* per-lane status bits HYK_LANE_* */
    /* persistent form only: the lanes to run, in the order they are taken
     * from the queue (lane_order[0..n_order), e.g. longest-first or the
     * active slots of a serving pool), or NULL for all lanes in index order */
    const uint64_t *lane_order;
    uint64_t n_order;
    /* optional checkpoint tape for the adjoint: the state (ck_capacity,
     * n_eq, ld), time (hi part) and step size (ck_capacity, ld) at the start
     * of every iteration; a lane that fills it stops with HYK_LANE_CAPACITY */
    double *ck_x;
    double *ck_t;
    double *ck_h;
    uint64_t ck_capacity;
    /* persistent form only: at most this many iterations per lane per call
     * (0 = until done).  A lane that reaches it is stored unfinished and the
     * next call continues it; used to time-slice a continuously refilled
     * batch (serving). */
    uint64_t slice_iters;
    /* events (modules with n_ev > 0): roots of non-terminal events are
     * recorded per lane, ev_t_hi/lo (ev_capacity, ld) = time of the root
     * (double-length), ev_info (ev_capacity, ld) = 4 * event index +
     * (direction + 1); ev_count (ld) = records so far (in/out).  A step whose
     * roots do not fit is not taken: the lane stops with HYK_LANE_CAPACITY.
     * ev_last (n_terminal, ld) = time of each terminal event's last trigger
     * (NaN: none; in/out, for the cooldown); ev_sign (ld) = direction of the
     * root of the terminal event that stopped a lane. */
    double *ev_t_hi;
    double *ev_t_lo;
    int32_t *ev_info;
    uint64_t *ev_count;
    uint64_t ev_capacity;
    double *ev_last;
    int32_t *ev_sign;
    /* optional: the reference's whole-batch stop on a non-finite state
     * (heyoka/expose_batch_integrators.cpp:279-314 returns err_nf_state for
     * the lane whose state became non-finite and stops every lane of the
     * batch at that iteration).  Device words of "iterations at which to
     * stop", one per group of stop_group lanes (stop_group 0: one word for
     * all lanes), initialised by the caller (UINT64_MAX: no stop).  A lane
     * whose state becomes non-finite at its iteration k lowers its group's
     * word to k (atomic minimum); a lane that has made as many iterations as
     * its group's word stops before its next one (HYK_LANE_STOPPED, its
     * outcome that of its last step).  The one-launch-per-step form steps the
     * unfinished lanes in lockstep, so one call gives the reference's result;
     * the persistent form runs lanes ahead of one another, so after a call
     * that lowered a word the caller restores the initial state and calls
     * again with the words as they were left.  NULL: every lane stops only
     * itself (per-lane semantics). */
    uint64_t *stop_iter;
    uint64_t stop_group;
} hyk_prop_t;

#define HYK_LANE_DONE 1u     /* reached the final time */
#define HYK_LANE_STOPPED 2u  /* stopped early: error, step limit, capacity or terminal event */
#define HYK_LANE_CAPACITY 4u /* stopped because tc_capacity, ck_capacity or ev_capacity was reached (resumable) */
#define HYK_LANE_EVENT 8u    /* stopped by a terminal event (propagation outcome = -(its index) - 1;
                                hyk_step reports the index itself) */

/* Initialise the bookkeeping arrays of `p` for a propagation to tf. */
int hyk_prop_init(hyk_module *m, const hyk_lanes_t *lanes, const hyk_prop_t *p, void *stream);

#define HYK_MODE_PLAIN 0      /* one kernel launch per step (drop-in form) */
#define HYK_MODE_PERSISTENT 1 /* persistent kernel, per-lane loops, lane queue */

/* Device workspace for hyk_propagate (bytes, 256-byte aligned pointer):
 * 256 bytes of counters, plus, for the PLAIN mode, a list of 8 bytes per
 * lane.  hyk_propagate accepts any workspace of at least
 * 256 bytes; with less than this size the PLAIN mode steps the lanes in
 * place instead of compacting the unfinished ones (same results, slower
 * when lanes finish at different times). */
size_t hyk_propagate_workspace_size(const hyk_module *m, uint64_t n_lanes, int mode);

/* Advance every unfinished lane until it is done or stopped.
 * PLAIN mode launches one step kernel per iteration (with a large enough
 * workspace, over a list of the unfinished lanes made before each launch)
 * and reads one word back every `check_every` launches to detect completion
 * (synchronises `stream`).
 * PERSISTENT mode runs one persistent launch.  `workspace` is device memory
 * of hyk_propagate_workspace_size() bytes.  On return, `*iters` (may be NULL)
 * holds the number of step launches made (PLAIN) or 1 (PERSISTENT). */
int hyk_propagate(hyk_module *m, const hyk_lanes_t *lanes, const hyk_prop_t *p, int mode,
                  void *workspace, size_t workspace_bytes, uint32_t check_every, uint64_t *iters,
                  void *stream);

/* hyk_propagate without a workspace, for callers that cannot allocate device
 * memory (code that runs inside another allocator's pool, a real-time loop
 * that must not allocate, a host integration without a CUDA allocator).  No
 * counterpart in the reference: it has no device memory at all.
 * The counters hyk_propagate keeps in its workspace live instead in one
 * file-scope device array of HYK_NOALLOC_SCRATCH_BYTES (4096) bytes, held by
 * every GPU that loads libhyk until the process exits.
 * The counters (256 bytes) always fit; the PLAIN mode compacts the
 * unfinished lanes when the lane list fits too (up to 480 lanes) and steps
 * the lanes in place otherwise.
 * The first call on a device looks up the array's device address; make that
 * first call before any stream capture.  Every call clears the counters it
 * needs before using them, so a call never sees the previous call's values,
 * but all calls share the one array: calls that overlap on the GPU (other
 * streams, other threads) race and give wrong results.  It allocates no
 * device memory and calls no allocating CUDA or library routine: the PLAIN
 * mode makes every launch directly (hyk_propagate replays its rounds as a
 * CUDA graph, which this entry point never creates or instantiates), and on
 * success no host memory is allocated either (an error message is the only
 * host allocation). */
#define HYK_NOALLOC_SCRATCH_BYTES 4096
int hyk_propagate_noalloc(hyk_module *m, const hyk_lanes_t *lanes, const hyk_prop_t *p, int mode,
                          uint32_t check_every, uint64_t *iters, void *stream);

/* Serving with a device work queue: one launch of a resident kernel that
 * integrates the lanes the caller appends to a device ring while it runs
 * (continuous batching without a relaunch per batch).  No counterpart in the
 * reference (heyoka.py has no server); it serves the same propagate_until
 * semantics per lane as hyk_propagate.  Lane form modules only.
 *   lanes, p: the pool's lane arrays and bookkeeping (as for hyk_propagate;
 *            n_lanes = the pool's capacity).  A lane is made ready by the
 *            caller writing its state, time, final time, bookkeeping
 *            (rem_hi/lo = final time - time, outcome, min_h = inf, max_h = 0,
 *            n_steps = n_iter = 0, status = 0) and owner, then its index at
 *            ring[tail % ring_capacity], then *tail = tail + 1, in that order
 *            on one stream (device copies only: while the kernel runs no
 *            other kernel can start on the SMs it holds).
 *   ring, ring_capacity (a power of two): the ring of lane indices;
 *   head: device word, the next ring position to take (advanced by the
 *         kernel; the caller initialises it once);
 *   tail: device word, the positions filled so far (advanced by the caller);
 *   stop: device word; non-zero makes idle threads return;
 *   owner: (ld) the request of each lane, an index into done_count;
 *   done_count: per request, the lanes finished so far (incremented by the
 *         kernel after the lane's results are stored and fenced);
 *   inflight: device word, lanes being integrated (0 before the first launch);
 *   status: device word receiving the HYK_SERVE_* reasons threads returned for;
 *   idle_ns: a thread without work returns after this long with an empty
 *         ring and no lane in flight; max_wait_ns: after this long waiting in
 *         any case (every wait of the kernel is bounded);
 *   grid_ctas: CTAs to launch (0: the GPU's resident capacity; a share of it
 *         lets the pools of several systems run their kernels side by side). */
typedef struct hyk_serve {
    uint64_t *ring;
    uint64_t ring_capacity;
    uint64_t *head;
    const uint64_t *tail;
    const uint32_t *stop;
    const int64_t *owner;
    uint32_t *done_count;
    uint64_t *inflight;
    uint32_t *status;
    uint64_t idle_ns;
    uint64_t max_wait_ns;
    uint32_t grid_ctas;
} hyk_serve_t;
#define HYK_SERVE_IDLE 1u    /* returned idle: empty ring, nothing in flight for idle_ns */
#define HYK_SERVE_STOP 2u    /* returned because *stop was set */
#define HYK_SERVE_TIMEOUT 4u /* a thread waited max_wait_ns for work while others still ran */
int hyk_serve(hyk_module *m, const hyk_lanes_t *lanes, const hyk_prop_t *p, const hyk_serve_t *s, void *stream);

/* Stream-ordered copy of `height` rows of `width` bytes between host and
 * device memory (pitches in bytes; either side may be host or device
 * memory): a copy-engine transfer, never a kernel, so that it runs while a
 * resident kernel holds the SMs (the serving pool's admissions and result
 * gathers). */
int hyk_memcpy2d(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, size_t height, void *stream);

/* Discrete adjoint of a taped propagation (module created with
 * HYK_CFG_ADJOINT).  For every lane, runs backwards over its n_steps[lane]
 * taped steps: recomputes the step's Taylor coefficients from the taped
 * state, then propagates the adjoint through the Horner update and the
 * Taylor recurrences in reverse, with the taped step sizes held fixed.
 *   lambda: (n_eq, ld) in: dL/dx(t_final); out: dL/dx(t_0)
 *   pbar:   (n_pars, ld) out: dL/dpars (NULL when n_pars == 0)
 *   lane_order: NULL (lanes in index order), or a permutation of
 *           0..n_lanes-1 in device memory, the order in which the threads
 *           take the lanes (longest tape first keeps the tail short);
 *           indices >= n_lanes are skipped
 * workspace: hyk_propagate_workspace_size() bytes, 256-byte aligned.
 * Gradient of the reference's propagation, which has no adjoint: no
 * counterpart in the reference (it offers forward variational equations,
 * heyoka/expose_var_ode_sys.cpp:29-59). */
int hyk_adjoint(hyk_module *m, const hyk_lanes_t *lanes, const double *ck_x, const double *ck_t, const double *ck_h,
                const int64_t *n_steps, const uint64_t *lane_order, double *lambda, double *pbar, void *workspace,
                size_t workspace_bytes, void *stream);

/* Dense output: out[i][l] = sum_n tc[i][n][l] * dt[l]^n (Horner), the
 * evaluator behind update_d_output / continuous output
 * (heyoka/expose_batch_integrators.cpp:519-541,
 *  heyoka/taylor_expose_c_output.cpp:272-408). */
int hyk_dense_eval(const double *tc, uint32_t n_eq, uint32_t order, uint64_t n_lanes, uint64_t ld,
                   const double *dt, double *out, void *stream);

/* Dense output of a single-precision module (float arrays, the same layout). */
int hyk_dense_eval_f32(const float *tc, uint32_t n_eq, uint32_t order, uint64_t n_lanes, uint64_t ld,
                       const float *dt, float *out, void *stream);

/* The deterministic elementary functions the kernels use, evaluated on the
 * device for validation: fn 0 exp, 1 log, 2 sin, 3 cos, 4 pow(x[i], a[i]),
 * 5 the step-size rho(m_p = x[i], m_pm1 = a[i], num = 1, order 20); 6..11 the
 * same functions in single precision (inputs rounded to float, order 9 for
 * rho), used by the float32 integrator.  x, a, out are device arrays of n doubles. */
int hyk_dmath_eval(int fn, const double *x, const double *a, double *out, uint64_t n, void *stream);

/* Device FP64 FMA throughput microbenchmark (flop/s, 2 flops per FMA), used
 * as the roofline denominator.  Runs for about `millis` milliseconds; uses a
 * one-double-per-CTA scratch buffer of its own. */
int hyk_fp64_peak(int device, double millis, double *flops_per_s);
/* The same probe in FP32 (the single-precision integrator's roofline). */
int hyk_fp32_peak(int device, double millis, double *flops_per_s);

/* Build check without a GPU: generate the module source for `d` at `order`
 * (block size cfg->block_lanes, default 128; the lane form with cold state
 * rows unless cfg->flags has HYK_CFG_NO_COLD_ROWS) and compile it with NVRTC
 * for sm_103a.  `log` receives the NVRTC log (ptxas register and spill
 * statistics when `verbose` is 1; the generated source, without compiling,
 * when `verbose` is 2; a host C++ translation unit of the same recurrences,
 * for CPU checks, when `verbose` is 3; the recurrences in the reference's
 * arithmetic over an element type the includer defines, the per-system part
 * of the compiled CPU stepper used as a timing baseline, when `verbose` is
 * 4); `n_slot` the shared-memory doubles per lane, `flops` the algorithmic
 * flops per step. */
int hyk_codegen_check(const hyk_decomp_t *d, uint32_t order, const hyk_config_t *cfg, int verbose, char *log,
                      size_t log_len, uint32_t *n_slot, double *flops);

const char *hyk_last_error(void);
const char *hyk_version(void);

#ifdef __cplusplus
}
#endif

#endif /* HYK_H */
