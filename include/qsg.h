/*
 * qsg.h -- C ABI of the GB300 split-operator engine (libqsg.so), and of its
 * Born-series scattering solvers (qsg_born_*, at the end of this file).
 *
 * Plain C, plain pointers and sizes; no exceptions cross it.  Every call
 * returns a qsg_status (0 = ok); qsg_last_error() gives the message of the
 * calling thread's last failure.
 *
 * It replaces, for the split-operator path of lhprojects/QuSim, what the
 * reference's evolver implementation does behind include/QuSim.h:
 *   - QuEvolverImpl / SplittingMethod1D / SplittingMethod2D
 *     (src/EvolverImpl.h:54-57, src/SplittingMethod1D.h, src/SplittingMethod2D.h)
 *   - its Device ops and FFT wrappers on the GPU_CUDA device
 *     (src/CudaDevice.cu:98-302, src/FourierTransform.cpp:84-127, 336-360)
 * A host evolver (include/qusim_gb300/Evolver.h, or a QuEvolverImpl subclass
 * inside the reference such as tests/cpp/ref_binding.cpp) drives it.
 *
 * Layout conventions are the reference's: complex values are interleaved
 * (re, im) doubles (std::complex<double>), a 2D grid is stored with index
 * iy + ix*ny (y contiguous; include/QuSim.h:47-52), and grid point i sits at
 * x0 + i*dx with dx = (x1 - x0)/n (src/EvolverImpl1D.cpp:11).
 *
 * Environment, read when a context is created (qsg_init):
 *   QSG_PLAN_CACHE      plan cache file of qsg_autotune / qsg_autotune_1d
 *                       (default ~/.cache/qusim_gb300/plans.tsv)
 *   QSG_COL_TMA=0       complex64 2D momentum-form column passes load their
 *                       tiles with load instructions instead of tensor copies
 *   QSG_FS_TMA=1        1D four-step column passes staged by tensor copies in
 *                       the default plans (off by default: measured slower on the
 *                       2048-instance batch; qsg_autotune_1d picks per size)
 *   QSG_BATCH_GRAPHS=1  batch steps replayed from captured CUDA graphs (off by
 *                       default: measured no faster)
 *   QSG_FAIL_PLAN_SWITCH=1  (read at each 1D plan switch) failure injection for
 *                       tests: a switch fails on the host after building the new
 *                       plan's tables, which are released again; the instance
 *                       keeps its plan
 * Every setting computes the same result bit for bit.
 * Read when a server is created (qsg_server_create):
 *   QSG_SERVER_FAIL_REQUEST=<id>  fault injection for tests of the failure
 *                       paths: every dispatch of request <id> fails on the host
 *                       with QSG_ERR_CUDA instead of launching (no device work
 *                       is faulted); the request ends failed and the other
 *                       requests run on unaffected
 *   QSG_SERVER_RING=<k> descriptor slots of the batched resident launches
 *                       (default 4096, at least max_running); tests set a small
 *                       ring so that its slots are reused many times over
 */
#ifndef QSG_H
#define QSG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    QSG_OK = 0,
    QSG_ERR_ARG = 1,          /* bad argument (null pointer, size, order ...)        */
    QSG_ERR_BUDGET = 2,       /* the request does not fit the context's HBM budget  */
    QSG_ERR_CUDA = 3,         /* a CUDA runtime error (message in qsg_last_error)   */
    QSG_ERR_TIMEOUT = 4,      /* a bounded device-side wait ran out                 */
    QSG_ERR_UNSUPPORTED = 5,  /* valid for the reference, not built here (e.g. a
                                 side above the supported lengths, InfiniteWall
                                 in 2D)                                             */
    QSG_ERR_STATE = 6         /* call not valid in the object's current state       */
} qsg_status;

typedef enum { QSG_FP64 = 0, QSG_MIXED = 1 } qsg_precision;
typedef enum { QSG_PERIOD = 0, QSG_INFINITE_WALL = 1 } qsg_boundary;

typedef struct qsg_ctx qsg_ctx;
typedef struct qsg_inst qsg_inst;

/* Library version string. */
const char *qsg_version(void);

/* Message of the calling thread's last failed call ("" if none). */
const char *qsg_last_error(void);

/* Open a context on CUDA device `device_ordinal`.  hbm_budget_bytes bounds the
 * device memory that instances of this context may hold (0 = no bound).
 * Replaces Device::Create(GPU_CUDA) (src/Device.cpp:24-33). */
int qsg_init(int device_ordinal, size_t hbm_budget_bytes, qsg_ctx **out);
void qsg_ctx_destroy(qsg_ctx *ctx);

/* The cudaStream_t every launch of this context goes to (as void*). */
void *qsg_ctx_stream(qsg_ctx *ctx);

/* Device bytes currently held by the context's instances and scratch. */
size_t qsg_ctx_bytes_in_use(qsg_ctx *ctx);

/* Create a 1D instance: n a power of two, 64 .. 8388608, or any other length
 * from 2 to 4194304, stepped through Bluestein transforms (as are the powers
 * of two below 64): in one CTA up to n = 4096, above that as two circular
 * convolutions of length M (the smallest power of two >= 2n - 1) on the
 * four-step passes over a buffer of M sites whose sites from n on stay zero.
 * psi0: n complex (re,im); V: n real (the reference keeps
 * only the real part of the potential, src/EvolverImpl1D.cpp:46).  dt is
 * complex (imaginary-time propagation allowed, include/QuSim.h:558-563).
 * order: 2 (SplittingMethodO2) or 4 (SplittingMethodO4).
 * boundary: QSG_PERIOD, or QSG_INFINITE_WALL (psi_0 = psi_n = 0, kinetic step
 * through the 2n odd extension, src/SplittingMethod1D.cpp:61-81): for powers
 * of two from 64, one CTA holds the 2n extension up to n = 4096 (QSG_MIXED) /
 * 2048 (QSG_FP64); above that, up to n = 4194304, the instance keeps the 2n odd
 * extension in HBM and steps it with the four-step passes of a periodic 2n
 * grid; any other n from 2 to 2048 keeps the 2n extension in one CTA stepped
 * by Bluestein transforms, and from 2049 to 2097152 steps it by Bluestein's
 * convolutions on the four-step passes (M >= 4n - 1).  Kept in HBM or in one
 * CTA, the extension's site 0 (the caller's psi_0) is zeroed before the first
 * step after each upload of the state (create, qsg_set_psi), site n is zero
 * from the upload on.  Reads and writes of psi cover its n sites.
 * Replaces SplittingMethod1D::InitSystem1D (src/SplittingMethod1D.cpp:5-31)
 * after the host has sampled psi0 / V (src/EvolverImpl1D.cpp:33-81). */
int qsg_create_1d(qsg_ctx *ctx, uint64_t n, double dx, double mass, double hbar,
                  double dt_re, double dt_im, int order, int precision, int boundary,
                  const double *psi0, const double *V, qsg_inst **out);

/* Create a 2D instance, nx*ny sites, index iy + ix*ny.  Periodic only, as in
 * the reference (src/SplittingMethod2D.cpp:21-29).  Sides that are powers of
 * two (128 .. 4096; nx = 8192 with ny up to 4096 in complex64, up to 2048 in
 * complex128; ny = 8192 with nx up to 4096 in complex64) run the split-k
 * passes with plans; a grid with a side that is not a power of two (each side
 * 2 .. 4096) runs row and column passes of Bluestein transforms.
 * Replaces SplittingMethod2D::InitSystem2D (src/SplittingMethod2D.cpp:5-31). */
int qsg_create_2d(qsg_ctx *ctx, uint64_t nx, uint64_t ny, double dx, double dy, double mass,
                  double hbar, double dt_re, double dt_im, int order, int precision,
                  const double *psi0, const double *V, qsg_inst **out);

/* Create a 3D instance, nx*ny*nz sites, index (ix*ny + iy)*nz + iz (z
 * contiguous, include/QuSim.h:54-61).  The reference has no 3D evolver, only
 * the 3D transform (src/FourierTransform.cpp:379-440) and a 3D kinetic
 * multiply; the step is SplittingMethod2D's (O2 / O4) with a third axis.
 * Sides: powers of two, 16 .. 1024, nz >= 16 (strided-pass tile width), at
 * most 2^30 sites.  qsg_step / qsg_norm2 / qsg_energies / qsg_get_psi /
 * qsg_set_psi work as for 1D and 2D. */
int qsg_create_3d(qsg_ctx *ctx, uint64_t nx, uint64_t ny, uint64_t nz, double dx, double dy, double dz,
                  double mass, double hbar, double dt_re, double dt_im, int order, int precision,
                  const double *psi0, const double *V, qsg_inst **out);

/* Initial state and potential given as a formula instead of arrays, sampled on
 * the device in FP64 at x_i = x0 + i*dx, y_j = y0 + j*dy (the points at which
 * the reference samples its psi / V functors, src/EvolverImpl1D.cpp:33-81,
 * src/EvolverImpl2D.cpp:39-98), so no host array is built or copied:
 *   psi0(r) = exp(i k.r) exp(-|r - c|^2 / (4 s^2)), scaled to
 *             sum |psi0|^2 dv = 1 when normalize (the reference's
 *             force_normalization);
 *   V(r)    = v0 + sum_b h_b exp(-|r - b_b|^2 / (2 w_b^2)), bumps[b] = {h, bx, by, w}.
 * In 1D the y terms (ky, cy, by) are unused.  This is the packet-plus-bumps
 * family of the benchmark and serving inputs; general expressions of the
 * reference's calculator language go through qsg_create_1d_expr /
 * qsg_create_2d_expr. */
#define QSG_SPEC_MAX_BUMPS 32
typedef struct {
    double x0, y0;
    double kx, ky;
    double cx, cy;
    double s;
    double v0;
    int32_t normalize;
    int32_t nbumps; /* 0 .. QSG_SPEC_MAX_BUMPS */
    double bumps[QSG_SPEC_MAX_BUMPS][4];
} qsg_spec;
/* qsg_create_1d / qsg_create_2d with psi0 and V from a spec (sampled into a
 * temporary device buffer of 24 bytes per site, counted against the HBM budget
 * while it lives). */
int qsg_create_1d_spec(qsg_ctx *ctx, uint64_t n, double dx, double mass, double hbar, double dt_re,
                       double dt_im, int order, int precision, int boundary, const qsg_spec *spec,
                       qsg_inst **out);
int qsg_create_2d_spec(qsg_ctx *ctx, uint64_t nx, uint64_t ny, double dx, double dy, double mass,
                       double hbar, double dt_re, double dt_im, int order, int precision,
                       const qsg_spec *spec, qsg_inst **out);

/* Initial state and potential as expressions in the language of the
 * reference's calculator (src/Cal.cpp: the strings FunctorWrapper /
 * Functor2DWrapper take, include/QuSim.h:502-538), sampled on the device in
 * complex128 at x_i = x0 + i dx (and y_j = y0 + j dy): numbers, x, y, Pi, I,
 * + - * / ^, comparisons < <= > >= == (real parts), && ||, c ? a : b, and sin
 * cos tan asin acos atan sinh tanh atanh exp log sqrt abs sign gauss(x, mu,
 * sigma).  V keeps the real part, as the reference does; psi0 is scaled to
 * sum |psi0|^2 dv = 1 when normalize (force_normalization).  A parse error
 * returns QSG_ERR_ARG with the message.  The samples pass through a temporary
 * device buffer of 24 bytes per site, counted against the HBM budget while it
 * lives.  Example (the double slit of the large 2D benchmark, without its
 * noise): "abs(x) < 1 ? (abs(y - 6) < 1 || abs(y + 6) < 1 ? 0 : 10) : 0". */
int qsg_create_1d_expr(qsg_ctx *ctx, uint64_t n, double x0, double dx, double mass, double hbar,
                       double dt_re, double dt_im, int order, int precision, int boundary,
                       const char *psi_expr, const char *v_expr, int normalize, qsg_inst **out);
int qsg_create_2d_expr(qsg_ctx *ctx, uint64_t nx, uint64_t ny, double x0, double y0, double dx,
                       double dy, double mass, double hbar, double dt_re, double dt_im, int order,
                       int precision, const char *psi_expr, const char *v_expr, int normalize,
                       qsg_inst **out);

/* Evaluate an expression of that language on the host (the reference's
 * Calculator::Evaluate, include/QuSim.h:527-538): nvars variables names[i]
 * with complex values values[2i], values[2i + 1]; *out = (re, im). */
int qsg_expr_eval(const char *expr, int nvars, const char *const *names, const double *values,
                  double *out);

/* Advance by nsteps steps (O2: V/2 T V/2; O4: the 7-factor Forest-Ruth
 * sequence), then, if renormalize, scale psi to Norm2 == 1.  Asynchronous:
 * returns once the launches are queued.  2D without renormalize: the last
 * pass of the call (closing V factor, back to natural layout) is deferred --
 * the next qsg_step opens with it merged into its own first pass, and every
 * call that reads the state (qsg_get_psi, qsg_norm2, qsg_energies, plan
 * changes) runs it first -- so a caller stepping in small calls pays no pass
 * more per step than one long call.
 * Replaces QuEvolverImpl::Step (src/EvolverImpl.cpp:56-68) with "batch" =
 * nsteps and force_normalization_each_step = renormalize, minus its device to
 * host copy of psi (qsg_get_psi does that on demand). */
int qsg_step(qsg_inst *inst, uint64_t nsteps, int renormalize);

/* Wait for the instance's queued work. */
int qsg_sync(qsg_inst *inst);

/* Norm2 = sum |psi|^2 dv (src/EvolverImpl.cpp:51-54). */
int qsg_norm2(qsg_inst *inst, double *out);

/* Norm2 of the state the last qsg_step left, as that step summed it: for a
 * 2D instance with real dt whose closing row pass is deferred (see qsg_step)
 * it is read from sums the step's last column pass took in split-k space,
 * with no pass over psi; otherwise it is qsg_norm2.  Equal to qsg_norm2 in
 * exact arithmetic (the closing V factor has modulus 1); in complex64 the
 * two sums differ by rounding (~1e-7 relative).  A per-step observable for
 * monitoring; qsg_norm2 is the reference's Norm2. */
int qsg_step_norm2(qsg_inst *inst, double *out);

/* The same value, read without stalling the stream: _post queues its sum and
 * a device-to-host copy after the work queued so far and returns a ticket;
 * _get waits for that copy only (later steps keep running) and returns the
 * value.  A loop can step, post, and collect the previous step's norm while
 * the current step runs.  The instance keeps the last 64 posts; older tickets
 * give QSG_ERR_STATE. */
int qsg_step_norm2_post(qsg_inst *inst, uint64_t *ticket);
int qsg_step_norm2_get(qsg_inst *inst, uint64_t ticket, double *out);

/* Kinetic and potential energy, as QuEvolverImpl::KinEn / PotEn
 * (src/SplittingMethod1D.cpp:91-107, src/SplittingMethod2D.cpp:123-138,
 * src/EvolverImpl.cpp:45-49).  Either pointer may be null. */
int qsg_energies(qsg_inst *inst, double *kin, double *pot);

/* <x> (src/EvolverImpl1D.cpp:83-88) and Norm2 over [xa, xb)
 * (src/EvolverImpl1D.cpp:90-102); 1D only.  x0 is the grid origin. */
int qsg_xavg(qsg_inst *inst, double x0, double *out);
int qsg_norm2_range(qsg_inst *inst, double x0, double xa, double xb, double *out);

/* Copy psi to the host as complex128 (n or nx*ny complex).  Synchronous. */
int qsg_get_psi(qsg_inst *inst, double *out);

/* Replace psi from a host complex128 array. */
int qsg_set_psi(qsg_inst *inst, const double *psi);

/* Steps taken so far (Time() = steps * dt, src/EvolverImpl.h:63-66). */
int qsg_steps_taken(qsg_inst *inst, uint64_t *out);

void qsg_destroy(qsg_inst *inst);

/* 2D execution plan: the x split (Nx = g * m, column transforms of length m,
 * a radix-g stage folded into the row pass), the elements per thread (radix)
 * of the row and column transforms, the threads per row-pass CTA, the
 * columns per column-pass CTA, and the row-pass kind (0: the unit of g rows
 * staged in shared memory; 1: one row per thread group in flight, the others
 * parked in the SM's tensor memory; complex64, g = 4, ny = 2048 or 4096).
 * Every plan computes the same result to rounding; they differ in speed.
 * New to this engine (the reference has one fixed cuFFT / KISS path). */
typedef struct {
    int32_t g;
    int32_t row_e;
    int32_t row_nt;
    int32_t col_e;
    int32_t col_w;
    int32_t row_kind;
} qsg_plan2d;

/* Plans compiled for an nx x ny grid at `precision`; fills up to cap, returns
 * the count (0 for an unknown precision or a grid without split-k plans). */
int qsg_candidate_plans(int precision, uint64_t nx, uint64_t ny, qsg_plan2d *out, int cap);
int qsg_get_plan(qsg_inst *inst, qsg_plan2d *out);
int qsg_set_plan(qsg_inst *inst, const qsg_plan2d *plan);

/* How a complex64 (QSG_MIXED) 2D instance holds its state between passes.
 * Both run the same passes of the reference's step (SplittingMethod2D,
 * src/SplittingMethod2D.cpp:81-121); they differ in rounding.
 *  QSG_FORM_MOMENTUM (default): the state is kept in momentum space,
 *    F psi / (nx ny), where the kinetic factor is a plain multiply; each
 *    potential factor is added as an increment, psi += F[(V - 1) F^-1 psi],
 *    so the FP32 rounding of its transforms scales with |V - 1| instead of
 *    with |psi|.  A column pass reads and writes the state beside its
 *    transform (32 instead of 16 bytes per site), and the instance holds one
 *    more nx*ny complex64 buffer.
 *  QSG_FORM_DIRECT: each pass transforms the state itself (16 bytes per site
 *    per pass); faster, about 2.5x the rounding error.
 * complex128 instances and 1D / 3D instances have one form (the direct one);
 * setting another returns QSG_ERR_UNSUPPORTED.  Setting the form runs any
 * deferred row pass first; the state itself is unchanged. */
typedef enum { QSG_FORM_MOMENTUM = 0, QSG_FORM_DIRECT = 1 } qsg_form;
int qsg_set_form(qsg_inst *inst, int form);
int qsg_get_form(qsg_inst *inst, int *form);

/* Failure-path check of the bounded device-side waits (no counterpart in the
 * reference).  Runs one column pass of a complex64 2D momentum-form instance
 * whose plan has the tensor-copy column pass (2048^2, 4096^2 plans) with its
 * tensor copies withheld: every CTA's first wait runs out after 1 s, sets the
 * context's error flag and returns before touching the state.  Returns the
 * status the following synchronisation reports: QSG_ERR_TIMEOUT when the path
 * works (the flag is then cleared and the context stays usable),
 * QSG_ERR_UNSUPPORTED for an instance without that pass. */
int qsg_check_wait_timeout(qsg_inst *inst);

/* Time every candidate plan for trial_steps steps on a copy of the
 * instance's state (psi and the step count are left unchanged), switch the
 * instance to the fastest, remember it for later instances of the same grid in
 * this context, and if persist append it to the plan cache file
 * ($QSG_PLAN_CACHE, default ~/.cache/qusim_gb300/plans.tsv) that new contexts
 * read.  Either out pointer may be null. */
int qsg_autotune(qsg_inst *inst, int trial_steps, int persist, qsg_plan2d *best,
                 double *best_ms_per_step);

/* 1D execution plan (no counterpart in the reference, whose periodic ExpT is
 * one FFT call each way per substep, src/SplittingMethod1D.cpp:40-60):
 *   kind 0: resident -- one CTA holds the whole line for the whole call
 *           (periodic n <= 8192 complex64 / 4096 complex128, one-CTA walls);
 *   kind 1: four-step -- two passes per substep over the n2 x n1 view of the
 *           line (n = n1 * n2, n from 8192 to 8388608, n1 a power of two from
 *           64 to 4096, n2 from 64 to 2048): column transforms of length n2, row transforms
 *           of length n1;
 *   tma:    four-step complex64 with n2 = 128 .. 512: the column pass stages
 *           its tiles with tensor copies instead of load instructions.
 * A wall above one CTA is stepped as its periodic 2n odd extension, so its
 * plans are the four-step plans of 2n (without tma).  Lengths that are not
 * powers of two (Bluestein) have one plan: kind 0 up to n = 4096 (a wall's
 * up to 2048), else kind 1 with the default split of M.  Every plan computes the
 * same result to rounding; they differ in speed.  New instances of a size
 * take the plan qsg_autotune_1d last chose for that size and precision in
 * this context or in the plan cache file, else the default (resident where
 * it fits, else four-step with n1 = n2 or 2 n2, load-instruction columns). */
typedef struct {
    int32_t kind;
    int32_t n1;
    int32_t tma;
    int32_t reserved;
} qsg_plan1d;

/* Plans for a 1D instance of n sites, `boundary` and `precision`; fills up to
 * cap (out may be null), returns the count (0: no instance of that shape). */
int qsg_candidate_plans_1d(int precision, uint64_t n, int boundary, qsg_plan1d *out, int cap);
int qsg_get_plan_1d(qsg_inst *inst, qsg_plan1d *out);
/* Switch an instance to another plan between steps (its state is kept).
 * QSG_ERR_UNSUPPORTED for a plan that is not a candidate, QSG_ERR_STATE for a
 * member of a batch (the batch's launches are built on its members' plans). */
int qsg_set_plan_1d(qsg_inst *inst, const qsg_plan1d *plan);
/* qsg_autotune for a 1D instance: every candidate plan timed for trial_steps
 * steps on a copy of the state (psi and the step count are left unchanged);
 * the instance switches to the fastest, which is remembered for new instances
 * of its size in this context and, if persist, appended to the plan cache file
 * ($QSG_PLAN_CACHE). */
int qsg_autotune_1d(qsg_inst *inst, int trial_steps, int persist, qsg_plan1d *best,
                    double *best_ms_per_step);

/* A batch of independent 1D instances of (possibly) different sizes, shared
 * order / precision / mass / hbar, per-instance dx, dt, psi0, V -- advanced
 * together.  Instances of one size are evolved by launches over all of them
 * (one CTA per instance for resident sizes, the four-step passes for the
 * others), each size on a stream of its own.  Each member is a qsg_inst owned
 * by the batch (qsg_batch_instance), usable with qsg_get_psi, qsg_norm2, ...
 * New to this engine (the reference evolves one system per Evolver). */
typedef struct qsg_batch qsg_batch;
int qsg_batch_create_1d(qsg_ctx *ctx, int count, const uint64_t *n, const double *dx, const double *dt_re,
                        const double *dt_im, double mass, double hbar, int order, int precision,
                        const double *const *psi0, const double *const *V, qsg_batch **out);
int qsg_batch_step(qsg_batch *batch, uint64_t nsteps);
int qsg_batch_sync(qsg_batch *batch);
int qsg_batch_size(qsg_batch *batch, int *count, uint64_t *sites);
int qsg_batch_instance(qsg_batch *batch, int i, qsg_inst **out);
void qsg_batch_destroy(qsg_batch *batch);

/* Plans of a batch's size classes (no counterpart in the reference).  A batch
 * is built on each size's cached plan (see qsg_plan1d); qsg_batch_autotune
 * tunes the four-step classes in the batch itself, because a launch over many
 * instances loads the GPU differently from one instance alone: each such class
 * is timed alone (all its members, at least trial_steps steps and 2^22
 * site-steps, on copies of their states, which are put back) on every
 * four-step plan of its length and keeps its fastest.  The choice stays with
 * the batch.  ms_per_step (may be null): the sum of the tuned classes' best
 * times per step.  qsg_batch_get_plan_1d / qsg_batch_set_plan_1d read and set
 * the plan of the members of length n (four-step plans only for four-step
 * classes; QSG_ERR_ARG for a length the batch does not hold). */
int qsg_batch_autotune(qsg_batch *batch, int trial_steps, double *ms_per_step);
int qsg_batch_get_plan_1d(qsg_batch *batch, uint64_t n, qsg_plan1d *out);
int qsg_batch_set_plan_1d(qsg_batch *batch, uint64_t n, const qsg_plan1d *plan);

/* Serving: evolution requests submitted as they arrive, run by a scheduler
 * thread with continuous batching under an HBM budget (new to this engine).
 * A request is a 1D (ny ignored) or 2D grid with its initial state, potential,
 * dt, step count and order; psi0 / V are copied at submit.  States: 0 queued,
 * 1 running, 2 done, 3 failed.  Requests are admitted first-in first-out while
 * the budget allows; running requests stay resident and advance in chunks, the
 * resident-size 1D ones of equal size batched into one launch; work of
 * different requests overlaps on the device.  A request's result does not
 * depend on what else runs. */
typedef struct qsg_server qsg_server;
typedef struct {
    int32_t dim;        /* 1 or 2 */
    int32_t order;      /* 2 or 4 */
    int32_t precision;  /* QSG_FP64 or QSG_MIXED */
    int32_t reserved;
    uint64_t nx, ny;
    double dx, dy, mass, hbar, dt_re, dt_im;
    uint64_t nsteps;
    const double *psi0; /* nx*ny complex */
    const double *V;    /* nx*ny real */
    const qsg_spec *spec; /* if not null, psi0 / V come from it (sampled on the device); copied at submit */
} qsg_request;
typedef struct {
    uint64_t completed, failed, site_steps;
    size_t peak_device_bytes, budget_bytes;
    uint64_t admitted_mid_flight; /* admissions made while other requests had work on the device */
    uint32_t max_in_flight;       /* most requests with device work queued (not yet finished) at once */
    uint32_t reserved;
} qsg_server_info;
/* One request's progress, times in seconds since the server was created
 * (-1: not reached yet).  Valid until qsg_server_take releases the request. */
typedef struct {
    int32_t state;               /* 0 queued, 1 running, 2 done, 3 failed */
    int32_t admitted_mid_flight; /* 1: admitted while other requests had work on the device */
    uint64_t chunks;             /* launches (or batched launches) made for it */
    uint64_t steps_dispatched;
    double t_submit, t_admit, t_first_dispatch, t_finish;
} qsg_request_info;
int qsg_server_create(int device_ordinal, size_t hbm_budget_bytes, int max_running, qsg_server **out);
int qsg_server_submit(qsg_server *server, const qsg_request *req, uint64_t *id);
int qsg_server_poll(qsg_server *server, uint64_t id, int *state);
int qsg_server_wait(qsg_server *server, uint64_t id, double timeout_s, int *state);
/* Copy the result (psi, complex128) and the submit-to-done latency; releases
 * the request.  A failed request returns its error here. */
int qsg_server_take(qsg_server *server, uint64_t id, double *psi_out, double *latency_s);
int qsg_server_stats(qsg_server *server, qsg_server_info *out);
int qsg_server_request_info(qsg_server *server, uint64_t id, qsg_request_info *out);
void qsg_server_destroy(qsg_server *server);

/* Per-kernel timing of this context's launches, for roofline reporting.
 * on = 1: CUDA events around every launch (they add a little time between
 * launches); on = 2: launch counts only, no events (total_ms stays 0); 0: off.
 * Enabling resets the counters.  qsg_profile_read fills up to cap entries of
 * name / launches / total milliseconds and returns the number of kernel kinds
 * seen. */
int qsg_profile_enable(qsg_ctx *ctx, int on);
int qsg_profile_read(qsg_ctx *ctx, int cap, const char **names, uint64_t *launches,
                     double *total_ms);

/* Norm2 of a wavefunction the caller already holds in device memory, computed
 * without allocating any device memory.  It has no counterpart in the
 * reference.
 *
 * For callers that cannot allocate: applications whose GPU memory is reserved
 * at start-up and handed out by another runtime's pool (a library cudaMalloc
 * fails there, or is not allowed), and real-time loops that may not call
 * cudaMalloc / cudaFree because those calls can stall the whole device.  It
 * needs no context and no instance.
 *
 * psi: n complex values on a CUDA device (complex128 for QSG_FP64, complex64
 * for QSG_MIXED), aligned to the element size.  *out = dv * sum |psi_i|^2,
 * written after the work queued on `stream` (a cudaStream_t on psi's device;
 * NULL = the default stream) has finished.  The call is synchronous: it waits
 * for that stream, so it cannot be made while the stream is being captured
 * into a graph (it returns QSG_ERR_STATE then); a stream of another device is
 * refused with QSG_ERR_ARG.
 *
 * Its scratch is one fixed 33,024-byte device array inside libqsg.so, which
 * every GPU that loads the library keeps until the process exits; n above
 * QSG_NORM2_NOALLOC_MAX_SITES (2^26) is rejected with QSG_ERR_ARG.  It calls
 * no cudaMalloc, cudaFree or other allocating routine.  The first call on each
 * device looks up the array's device address (cudaGetSymbolAddress).  All calls on a device share
 * the one array: calls that overlap on the GPU (different streams, or host
 * threads not ordered with each other) race and can return wrong sums. */
#define QSG_NORM2_NOALLOC_MAX_SITES 67108864ull
int qsg_norm2_noalloc(const void *psi, uint64_t n, int precision, double dv, void *stream,
                      double *out);

/* ------------------------------------------------------------------------
 * Born-series scattering solvers: QuPerturbation1D / QuPerturbation2D
 * (include/QuSim.h:689-806; src/Perturbation1DImpl.cpp, src/Perturbation2DImpl.cpp,
 * src/Perburbation.h, src/ScatteringSolverImpl.cpp).  A solver holds the
 * incident wave psi0 = exp(i k0 d.r) (k0 = sqrt(2 m E) / hbar, d the unit
 * direction), the potential V (complex, as the reference's functor returns
 * it) and the scattered part psi of the wave function; each qsg_born_compute
 * runs `order` updates of the naive or the preconditioned series on psi.
 * Grids: 1D n a power of two, 128 .. 2^22; 2D nx, ny powers of two,
 * 64 .. 4096 (other sizes: QSG_ERR_UNSUPPORTED).
 * ------------------------------------------------------------------------ */
typedef struct qsg_born qsg_born;

/* the "preconditioner" option values (src/PerturbationOptions.cpp:15-31);
 * QSG_BORN_IDENTITY is the reference's "BornIndentity" */
typedef enum {
    QSG_BORN_IDENTITY = 0,
    QSG_BORN_VELLEKOOP = 1,
    QSG_BORN_HAO1 = 2,
    QSG_BORN_HAO2 = 3
} qsg_born_preconditioner;

/* the reference's Options keys for these solvers (PerturbationCommon,
 * src/PerturbationOptions.cpp:8-43); qsg_born_default_opts gives its defaults */
typedef struct {
    int order;           /* "order": updates per compute (default 1; >= 1 here)          */
    int preconditional;  /* "preconditional": 0 naive series, 1 preconditioned          */
    int preconditioner;  /* "preconditioner" (default QSG_BORN_VELLEKOOP)                */
    double slow;         /* "slow" (default 1)                                           */
} qsg_born_opts;
void qsg_born_default_opts(qsg_born_opts *opts);

/* QuPerturbation1D::init (src/Perturbation1DImpl.cpp:7-42): grid x_i = x0 + i dx,
 * dx = (x1 - x0) / n; V: n complex (re, im) sampled there; en the energy;
 * epsilon the i eps of the Green's function (raised to the preconditioner's
 * minimum when preconditioned); direction > 0 right-going, else left-going.
 * The preconditioned series adds the reference's absorbing layer to Im V and
 * needs a box of at least 24 wavelengths (QSG_ERR_ARG otherwise). */
int qsg_born_create_1d(qsg_ctx *ctx, uint64_t n, double x0, double x1, const double *V, double en,
                       double epsilon, double direction, double mass, double hbar,
                       const qsg_born_opts *opts, int precision, qsg_born **out);
/* QuPerturbation2D::init (src/Perturbation2DImpl.cpp:4-47): V nx*ny complex,
 * index iy + ix*ny; (dirx, diry) the incident direction (normalised here). */
int qsg_born_create_2d(qsg_ctx *ctx, int nx, int ny, double x0, double x1, double y0, double y1,
                       const double *V, double en, double epsilon, double dirx, double diry,
                       double mass, double hbar, const qsg_born_opts *opts, int precision,
                       qsg_born **out);
/* Compute(): `order` updates; then (1D) R and T, (2D) the delta-psi norm.
 * Queued on the context's stream; the results below wait for it. */
int qsg_born_compute(qsg_born *b);
/* GetPsi / GetPsi0 / GetV: what = QSG_BORN_PSI (the scattered part), QSG_BORN_PSI0
 * or QSG_BORN_V (with the absorbing layer); out: n complex (re, im). */
typedef enum { QSG_BORN_PSI = 0, QSG_BORN_PSI0 = 1, QSG_BORN_V = 2 } qsg_born_field;
int qsg_born_get(qsg_born *b, int what, double *out);
/* GetR / GetT (1D), after a compute (ScatteringSolver1DImpl::ComputeRT) */
int qsg_born_rt(qsg_born *b, double *R, double *T);
/* GetDeltaPsiNorm (2D): sqrt(sum |psi - psi_before|^2 / sum |psi|^2) of the last compute */
int qsg_born_delta_norm(qsg_born *b, double *out);
/* GetEpsilon: the epsilon in use */
int qsg_born_epsilon(qsg_born *b, double *out);
/* ComputeXSection (2D) for `count` directions cosxy[2*i], cosxy[2*i+1]: out[i] */
int qsg_born_xsection(qsg_born *b, int count, const double *cosxy, double *out);
/* ComputeTotalXSection(n) (2D): sum over theta_i = 2 pi i / n of the
 * cross section, times 2 pi / n */
int qsg_born_total_xsection(qsg_born *b, int n, double *out);
void qsg_born_destroy(qsg_born *b);

#ifdef __cplusplus
}
#endif

#endif /* QSG_H */
