/*
 * montjoie_gb300 - C ABI of the GB300 matrix-free acoustic operator and
 * leap-frog time loop.
 *
 * Drop-in boundary for one hot path of Montjoie (marcdurufle33/Montjoie): the
 * matrix-free stiffness product of the scalar acoustic (Laplace) equation on
 * mass-lumped Gauss-Lobatto Q_r hexahedra, and the order-2 leap-frog
 * (ModifiedEquationIterator) that drives it.  Plain pointers and sizes only;
 * every call returns MJ_OK (0) or an error code and never aborts; the text of
 * the last error of the calling thread is returned by mj_last_error().
 *
 * Array conventions (the reference's):
 *  - Nodle: n_elt x (r+1)^3 int32 global dof numbers, row e in the reference
 *    local order NumDofs3D (vertices, edges, faces, interior;
 *    MONTJOIE/src/Quadrature/HexahedronQuadrature.cxx:51-171);
 *  - stiffness factors: n_elt x (r+1)^3 x 6 doubles, the symmetric 3x3
 *    B = (J w) DF^-1 mu DF^-T of every quadrature point (= dof) in local order,
 *    entries xx, xy, xz, yy, yz, zz (Glob_matMass_Bh,
 *    MONTJOIE/src/Elliptic/Helmholtz/VarHelmholtz.cxx:95-123);
 *  - 1-D rule: Gauss-Lobatto points on [0,1] and G[a*(r+1)+b] = phi_a'(x_b)
 *    (Globatto::ComputeGradPhi, MONTJOIE/src/Quadrature/GaussLobatto.cxx:175-191).
 * All vectors are contiguous arrays of n_dof doubles (Seldon Vector<double>
 * storage, GetData()).
 */
#ifndef MONTJOIE_GB300_H
#define MONTJOIE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------- */
#define MJ_OK 0
#define MJ_ERR_ARG 1         /* invalid argument (size, range, null pointer) */
#define MJ_ERR_CUDA 2        /* a CUDA call failed (text in mj_last_error) */
#define MJ_ERR_STATE 3       /* call out of order (e.g. advance before init) */
#define MJ_ERR_NONFINITE 4   /* non-finite value met (divergence guard) */
#define MJ_ERR_GEOMETRY 5    /* non-positive Jacobian (degenerate element) */
#define MJ_ERR_NOMEM 6       /* device allocation failed */

/* ---- precision of an operator ---------------------------------------- */
#define MJ_FP64 0   /* plain form: FP64 everywhere */
#define MJ_FP32 1   /* chosen form: FP32 state, factors and contractions,
                       FP64 setup, mass inversion and diagnostics */

typedef struct mj_op mj_op;
typedef struct mj_lf mj_lf;

/* Returns the message of the last failed call on this thread ("" if none). */
const char* mj_last_error(void);

/* Library version string. */
const char* mj_version(void);

/* ---- operator -------------------------------------------------------- */

typedef struct {
  int order;          /* r >= 1, r <= 8 */
  int n_elt;          /* number of hexahedra */
  int n_dof;          /* number of global dofs */
  const int32_t* nodle;   /* n_elt x (r+1)^3, host memory */
} mj_mesh_desc;

typedef struct {
  const double* factors;   /* n_elt x (r+1)^3 x 6, host memory */
  const double* gradphi;   /* (r+1)^2 derivative matrix, or NULL: built from the GL rule */
} mj_geom_desc;

/* Creates the operator y <- beta*y + alpha*A*x on the current CUDA device.
 * Replaces the construction of FemMatrixFreeClass<double, LaplaceEquation<Dimension3> >
 * (MONTJOIE/src/Computation/FemMatrixFreeClass.hxx:74-300; its data is the
 * problem's Nodle and Glob_matMass_Bh). precision: MJ_FP64 or MJ_FP32. */
int mj_op_create(const mj_mesh_desc* mesh, const mj_geom_desc* geom, int precision, mj_op** out);

/* Creates the same operator from the mesh's geometry instead of host factors:
 * the FP64 stiffness factors B = (J w) DF^-1 mu_e DF^-T of straight-sided
 * (trilinear) hexahedra are computed on the device directly in the
 * operator's layout (VarGeometryProblem.cxx:685-759, VarHelmholtz.cxx:54-131;
 * the arithmetic of mj_geometry, so the factors are the same bits), and the
 * vertices stay on the device for mj_op_lumped_mass and mj_op_gaussian_source.
 * verts: n_elt x 8 x 3 host (reference-cube vertex order); mu: n_elt host.
 * MJ_ERR_GEOMETRY when a Jacobian is not positive.  No reference counterpart
 * as one call: it replaces the setup of Glob_matMass_Bh plus
 * FemMatrixFreeClass construction. */
int mj_op_create_geometry(const mj_mesh_desc* mesh, const double* verts, const double* mu, int precision,
                          mj_op** out);

/* Lumped mass D_i = sum over the points on dof i of rho_e J w, assembled on
 * the device in element order (the reference's assembly order,
 * ContinuousMassMatrixAcoustic::Init, TimeAcoustic.cxx:889-965, so the sums
 * round as the host loop's; the same bits as mj_lumped_mass for rho = 1).
 * rho: n_elt host values, or NULL (1; then D is also the norm weight sum of
 * J w of GetNormeSolution).  mass_out: n_dof host.  Operators from
 * mj_op_create_geometry only (MJ_ERR_STATE otherwise). */
int mj_op_lumped_mass(mj_op* op, const double* rho, double* mass_out);

/* Gaussian volume source F_i = sum over the points on dof i of J w g(x),
 * g = beta exp(-alpha r^2) for r = |x - center| < radius, alpha =
 * -ln(1e-6)/radius^2, beta = sqrt(alpha/pi) (GaussianSource::GetAmplitude,
 * MONTJOIE/src/Source/SourceSpatiale.cxx:78-90; the right-hand side of
 * VarInstationary.cxx:620-676), assembled on the device in element order.
 * Returns the non-zero entries in increasing dof order: *n_out of them, the
 * first `capacity` in idx_out / val_out (both may be NULL to count only;
 * MJ_ERR_ARG when they do not fit).  Operators from mj_op_create_geometry. */
int mj_op_gaussian_source(mj_op* op, const double* center, double radius, int capacity, int32_t* idx_out,
                          double* val_out, int* n_out);

/* Largest eigenvalue of D^-1 A by power iteration on the device, for the
 * explicit time step dt = C / sqrt(lambda) (the reference's TimeStep = AUTO
 * needs ARPACK/SLEPc, EvaluationCflWave.cxx:729-741): x_0 = x0 (host, n_dof),
 * y = D^-1 A x_k in the operator's precision (as mj_op_mltadd computes it),
 * lambda = |y| / |x_k|, x_{k+1} = y / |y|, iters times. */
int mj_op_power_iteration(mj_op* op, const double* inv_mass, const double* x0, int iters, double* lambda_max);

/* Releases every device buffer of the operator. NULL is accepted. */
int mj_op_destroy(mj_op* op);

/* y <- beta*y + alpha*A*x with HOST vectors of n_dof doubles (y is not read when
 * beta == 0).  Replaces VirtualMatrix<double>::MltAddVector(alpha, x, beta, y)
 * (SELDON/matrix/Matrix_Base.hxx:41-140) as implemented by
 * FemMatrixFreeClass_Base<T>::MltAddVector (MONTJOIE/src/Computation/FemMatrixFreeClass.cxx:953-1166)
 * and MltAddScalarH1 (MONTJOIE/src/Computation/ProdMatVectScalarH1.cxx:679-727).
 * Synchronous. */
int mj_op_mltadd(mj_op* op, double alpha, const double* x, double beta, double* y);

/* Same product on DEVICE vectors of n_dof elements in the operator's precision
 * (double for MJ_FP64, float for MJ_FP32), ordered on `stream`
 * (a cudaStream_t, NULL = legacy default stream).  Asynchronous. */
int mj_op_mltadd_device(mj_op* op, double alpha, const void* x, double beta, void* y, void* stream);

/* Sizes and layout facts of an operator. */
int mj_op_info(const mj_op* op, int* order, int* n_elt, int* n_dof, int* precision,
               size_t* device_bytes);

/* Element-kernel variant chosen by the autotuner at creation: elements per
 * CTA, work layout (0 compact, 1 vector lines, 2 one element per warp, 3 one
 * element per warp reading the packed connectivity: each point's dof with its
 * rank among the dof's elements, so the result slot is the dof's CSR offset
 * plus the rank and no slot array is read; 4 compact with one factor stage:
 * the next tile's factors are copied during the current tile's divergence,
 * so a CTA holds one factor block instead of two), grid; and the timings (ms per launch,
 * or a negative occupancy score on meshes too small to time) of the
 * candidates tried (candidate_ms may be NULL, else room for 64 values). */
int mj_op_tuning(const mj_op* op, int* tile_elems, int* vector_lines, int* grid, int* n_candidates,
                 double* candidate_ms);

/* Forces the element-kernel variant instead of the autotuner's choice:
 * tile_elems elements per CTA and the work layout (vector_lines: 0 compact,
 * 1 vector lines, 2 one element per warp, 3 the same with packed
 * connectivity, 4 compact with one factor stage; 1 to 4 are FP32 only, 2 and
 * 3 exist for order 4, 3 for meshes of fewer than 2^27 dofs each shared by
 * at most 32 elements);
 * MJ_ERR_ARG when no such variant exists for the order.  Integrators bound to the operator
 * keep captured CUDA graphs of the old variant until re-created. */
int mj_op_set_variant(mj_op* op, int tile_elems, int vector_lines);

/* Number of kernels this library launched on the calling process since load. */
uint64_t mj_kernel_launches(void);

/* Test hook, no reference counterpart.  Every wait of the library's kernels
 * is bounded: on a bulk copy (mbarrier), 2^22 polls; on the other CTAs of a
 * cooperative launch (grid barrier), barrier_polls polls (default 2^26) or
 * barrier_ns nanoseconds (default 2 s), whichever comes first.  A wait that
 * runs out makes the kernel report through its error flag after letting its
 * own copies in flight land, and the entry point returns MJ_ERR_CUDA (element
 * kernels) or MJ_ERR_STATE (cooperative steps) with a message; the state is
 * then invalid but the next call starts clean.  This call lets a test make
 * waits run out: mbar_polls = 0 switches two element-kernel variants (FP32
 * one element per warp, order 4, 2 elements per CTA; FP64 compact, order 4,
 * 4 elements per CTA; see mj_op_set_variant) to instances compiled with a
 * bulk-copy wait limit of 0 (the bound is a compile-time constant in the
 * kernels), any other value switches them back; barrier_polls and
 * barrier_ns lower the grid barrier's limits (0: give up after the first
 * poll; values above the defaults are clamped to them; negative values
 * restore them).  Process-wide; captured CUDA graphs keep the kernels they
 * were captured with. */
int mj_debug_set_wait_limits(long long mbar_polls, long long barrier_polls, long long barrier_ns);

/* ---- leap-frog time loop -------------------------------------------- */

typedef struct {
  double dt;                 /* time step */
  const double* mass;        /* lumped mass D (n_dof), host */
  const double* inv_mass;    /* 1/D as the scheme uses it (n_dof), host; NULL -> 1/D */
  int n_src;                 /* sparse spatial source F: n_src (index, value) pairs */
  const int32_t* src_idx;
  const double* src_val;
  int n_pulse;               /* pulse p(t_n + dt) of step n = 0..n_pulse-1, host; */
  const double* pulse;       /* steps past n_pulse get no source */
  const double* norm_weight; /* per-dof weight M_i = sum of J*w over the points on
                                dof i (n_dof), or NULL: no norm diagnostics */
  int n_rec;                 /* receivers: n_rec x n_rec_w (dof, weight) pairs */
  int n_rec_w;
  const int32_t* rec_idx;
  const double* rec_w;
} mj_lf_desc;

/* Binds a leap-frog integrator to an operator (copies the descriptor's arrays
 * to the device).  Replaces ModifiedEquationIterator<double> of order 2
 * (MONTJOIE/src/Instationary/ModifiedEquation.hxx:78-114) with its
 * VirtualOdeSystem operators ApplyOperatorKh/Dh/DhMinusdtSh, SolveOperatorDhPlusdtSh
 * and AddScalarTimeSource (MONTJOIE/src/Instationary/TimeSchemes.hxx:35-151). */
int mj_lf_create(mj_op* op, const mj_lf_desc* desc, mj_lf** out);
int mj_lf_destroy(mj_lf* lf);

/* Initial conditions U^0 = u0, U^1 = U^0 + dt*(du0 + dt/2 * D^-1(-A U^0))
 * (ModifiedEquationIterator::SetInitialConditionS,
 *  MONTJOIE/src/Instationary/ModifiedEquation.cxx:92-124).  Host vectors;
 * du0 may be NULL (zero).  Resets the step counter to 0. */
int mj_lf_init(mj_lf* lf, const double* u0, const double* du0);

/* Advances nsteps steps (Advance, ModifiedEquation.cxx:290-345).  Before each
 * step the iterate U^n is handed to the diagnostics, as GiveIterate is
 * (ModifiedEquation.cxx:40-47): norms[s] (if not NULL, nsteps entries) gets
 * sum_i M_i u_i^2 (GetNormeSolution, VarInstationary.cxx:2696-2745) and
 * traces[k*trace_stride + s] (if not NULL) the receiver values.  Host outputs. */
int mj_lf_advance(mj_lf* lf, int nsteps, double* norms, double* traces, int trace_stride);

/* Copies U^n (the current iterate) and U^{n+1} to host vectors (either may be NULL). */
int mj_lf_get_state(mj_lf* lf, double* u_n, double* u_np1);

/* Whole run of RunSecondOrderScheme (ModifiedEquation.cxx:16-53): init from
 * host u0/du0, nsteps steps with diagnostics of U^0..U^{nsteps-1}, then the
 * final iterate U^{nsteps} (GiveFinalIterate) into u_final and, when norms /
 * traces are given, its diagnostics in entry nsteps (norms: nsteps+1 entries,
 * trace_stride >= nsteps+1).  Host buffers; synchronous. */
int mj_lf_run(mj_lf* lf, const double* u0, const double* du0, int nsteps, double* u_final,
              double* norms, double* traces, int trace_stride);

/* Device-side access for callers that keep the state resident: pointers to the
 * current U^n and U^{n+1} buffers (operator precision) and the step counter. */
int mj_lf_device_state(mj_lf* lf, void** u_n, void** u_np1, int* step);

/* Per-kernel device time of the steps run by mj_lf_advance / mj_lf_run while
 * enabled (CUDA events on the integrator's stream around the element kernel
 * and the gather/update kernel; the first 1024 steps of each call are timed).
 * enable = 1 resets the totals and starts timing, 0 stops it; the current
 * totals are returned in every case.  No reference counterpart (the
 * reference's phase timers, MONTJOIE/src/Share/Timer.hxx:14-23, play this role). */
int mj_lf_profile(mj_lf* lf, int enable, double* elem_ms, double* update_ms, int* steps);

/* mj_lf_advance replays a captured CUDA graph of 20 steps (two kernels per
 * step) when it records no diagnostics and profiling (mj_lf_profile) is off;
 * enable = 0
 * launches every kernel from the host instead.  Default: enabled. */
int mj_lf_set_graph(mj_lf* lf, int enable);

/* Time scheme of the integrator: order 2 (the leap-frog, default) or order 4,
 * the modified-equation leap-frog of ModifiedEquationIterator with order 4
 * (MONTJOIE/src/Instationary/ModifiedEquation.cxx:125-175 start, :346-408
 * step; no damping term).  Order 4 takes two stiffness products per step and
 * allows a CFL constant of 2 sqrt(3) instead of 2 (:217-225).  pulse_d2: the
 * second time derivative of the pulse at t_n + dt for n = 0..n_pulse_d2-1
 * (derivative order 3 of the source primitive, TimeSource.cxx:826-880), host.
 * Call before mj_lf_init; the iterate handed out and returned is u(t_n) as
 * for order 2. */
int mj_lf_set_scheme(mj_lf* lf, int order, int n_pulse_d2, const double* pulse_d2);

/* FP32 order-2 step: with enable != 0 (the default for MJ_FP32) the gather,
 * update and source run as one streaming kernel that stages each chunk of
 * dofs (states, dt^2/D, CSR offsets, contributions) in shared memory by bulk
 * copy; enable = 0 uses a gather kernel and a separate source kernel.  Both
 * give the same states bit for bit. */
int mj_lf_set_stream_gather(mj_lf* lf, int enable);

/* Divergence guard: mj_lf_advance / mj_lf_run return MJ_ERR_NONFINITE (with
 * the offending value in mj_last_error) when a recorded norm exceeds
 * norm_max in absolute value, or is not finite.  The reference checks
 * |GetNormeSolution| against NormeMaxSolution (default 1e30, the default
 * here too) and aborts (MONTJOIE/src/Instationary/VarInstationary.cxx:362-374,
 * 2741-2745); here the call returns after its chunk of steps, the norms up to
 * the offending step being valid.  Norms are only computed when asked for. */
int mj_lf_set_norm_max(mj_lf* lf, double norm_max);

/* Sets the CUDA stream (cudaStream_t) used by the integrator's launches. */
int mj_lf_set_stream(mj_lf* lf, void* stream);

/* ---- many sources on one mesh ------------------------------------------ */

typedef struct mj_lfb mj_lfb;

typedef struct {
  double dt;                 /* time step */
  int n_rhs;                 /* S independent runs (one per source), multiple of 8, <= 4096 (the Python
                                BatchLeapFrog pads other counts with runs that have no source) */
  const double* mass;        /* lumped mass D (n_dof), host */
  const double* inv_mass;    /* 1/D (n_dof), host; NULL -> 1/D */
  int n_src;                 /* sparse sources: entry t adds pulse * src_val[t] at dof */
  const int32_t* src_idx;    /* src_idx[t] of run src_rhs[t] */
  const int32_t* src_rhs;
  const double* src_val;
  int n_pulse;               /* pulse p(t_n + dt) shared by all runs, host */
  const double* pulse;
  int n_rec;                 /* receivers sampled for every run: n_rec x n_rec_w (dof, weight) */
  int n_rec_w;
  const int32_t* rec_idx;
  const double* rec_w;
} mj_lfb_desc;

/* Binds S leap-frog runs that share the mesh (and the operator, which must be
 * MJ_FP32) but have their own sources and states; the state lives on the
 * device as an n_dof x S array (row-major: the S values of a dof together).
 * Each run is the order-2 ModifiedEquationIterator of mj_lf_create
 * (MONTJOIE/src/Instationary/ModifiedEquation.cxx:92-124,290-345); the
 * reference runs them one after the other.  The element-kernel variant is
 * chosen by timing the candidates on this operator. */
int mj_lfb_create(mj_op* op, const mj_lfb_desc* desc, mj_lfb** out);
int mj_lfb_destroy(mj_lfb* b);

/* U^0 = u0, U^1 from SetInitialConditionS for every run; u0, du0: n_dof x S
 * host arrays (row-major), NULL = zero. */
int mj_lfb_init(mj_lfb* b, const double* u0, const double* du0);

/* Advances nsteps steps of every run.  use_graph != 0 replays a captured
 * CUDA graph of 20 steps (two kernels per step) when no traces are asked.
 * traces (or NULL): receiver k of run s before step j of this call at
 * traces[(k*S + s)*trace_stride + j]. */
int mj_lfb_advance(mj_lfb* b, int nsteps, double* traces, int trace_stride, int use_graph);

/* Copies U^n and U^{n+1} (n_dof x S row-major, either may be NULL) to the host. */
int mj_lfb_get_state(mj_lfb* b, double* u_n, double* u_np1);

/* Tuned variant and progress: runs, elements per CTA, lanes (runs per pass), grid, steps done. */
int mj_lfb_info(const mj_lfb* b, int* n_rhs, int* tile_elems, int* lanes, int* grid, int* step);

/* mj_lfb_advance runs every step as ONE cooperative persistent kernel
 * (element products of all runs, grid barrier, gather + update + sources),
 * its variant chosen at creation by timing the candidates of the order; with
 * enable = 0 it uses two kernels per step (element kernel, then gather and
 * update) instead.  Default: one kernel when a variant fits (MJ_ERR_STATE
 * otherwise). */
int mj_lfb_set_fused(mj_lfb* b, int enable);

/* One-kernel step: whether it is in use, threads per CTA and grid of the
 * chosen variant, and the timings (ms per step) of the candidates tried
 * (candidate_ms: room for 16, may be NULL). */
int mj_lfb_step_info(const mj_lfb* b, int* fused, int* threads, int* grid, int* n_candidates, double* candidate_ms);

/* Forces the one-kernel step's variant instead of the timed choice:
 * tile_elems elements per tile; lanes thread lanes per z-line of an element
 * (lanes x sources_per_thread right-hand sides per pass); sources_per_thread
 * right-hand sides held by each thread.  Every variant gives the same states
 * bit for bit.  MJ_ERR_ARG when no such variant exists for the order or the
 * number of right-hand sides. */
int mj_lfb_set_step_variant(mj_lfb* b, int tile_elems, int lanes, int sources_per_thread);

/* Profiling aid for the one-kernel step: with enable != 0 every step is a
 * plain launch recording per-CTA time stamps; mj_lfb_phase_ms then returns,
 * for the last step, out[0] = element phase (last CTA), out[1] = element phase
 * (mean CTA), out[2] = barrier release, out[3] = dof phase, in ms. */
int mj_lfb_profile(mj_lfb* b, int enable);
int mj_lfb_phase_ms(const mj_lfb* b, double* out);

/* ---- many meshes of different size and order --------------------------- */

typedef struct mj_mb mj_mb;

/* Groups n_runs leap-frog runs into one batch.  Each run comes from
 * mj_lf_create on its own MJ_FP32 operator, with its own mesh, order (1..8),
 * time step, mass, source and pulse.  Every time step of every run is ONE
 * cooperative persistent kernel: the element products of all meshes, a
 * grid-wide barrier, then the gather, update and source of all meshes.
 * Each run keeps its own state.  Between calls it stays usable through
 * mj_lf_init, mj_lf_advance and mj_lf_get_state.  Runs must not share an
 * operator.  The reference advances such runs one after the other, each
 * with its own ModifiedEquationIterator
 * (MONTJOIE/src/Instationary/ModifiedEquation.cxx:290-345). */
int mj_mb_create(int n_runs, mj_lf* const* runs, mj_mb** out);
int mj_mb_destroy(mj_mb* mb);

/* Advances every run by nsteps steps; every run must have been initialised
 * (mj_lf_init).  use_graph != 0 replays a captured CUDA graph of 20 steps.
 * Every run needs the order-2 scheme (not mj_lf_set_scheme order 4).  The
 * batch must be destroyed before its runs. */
int mj_mb_advance(mj_mb* mb, int nsteps, int use_graph);

/* Launch shape of the batch kernel: CTAs, CTAs per SM, element tiles and dof
 * chunks per step, 1 if the last advance replayed a graph, and the order
 * index n = r+1 when every mesh has that order (the batch then runs the
 * kernel instance of that order alone), else 0.  Grouped by order
 * (mj_mb_grouping): tiles and chunks of all groups, CTAs of the largest
 * group.  A union (mj_mb_union_info): its element kernel's CTAs and tiles
 * and its streaming gather's chunks.  Any output may be NULL. */
int mj_mb_info(const mj_mb* mb, int* grid, int* ctas_per_sm, int* n_tiles, int* n_chunks, int* graph,
               int* single_order);

/* Profiling aid: with enable != 0 every step is a plain launch that records
 * per-CTA time stamps; mj_mb_phase_ms then returns, for the last step (out:
 * room for 6), out[0] = element phase (last CTA), out[1] = element phase
 * (mean CTA), out[2] = barrier release, out[3] = dof phase, out[4] = time a
 * CTA spent waiting for its element tiles' bulk copies, out[5] = the same for
 * its dof chunks (means over the CTAs), in ms. */
int mj_mb_profile(mj_mb* mb, int enable);
int mj_mb_phase_ms(const mj_mb* mb, double* out);

/* Launch configuration of the batch kernel, timed on the batch at its first
 * advance (run states are restored afterwards): threads per CTA (256: large
 * tiles, 128: small tiles, more CTAs per SM; 0 before the first advance) of
 * the configuration in use, or of the faster one when another form runs
 * (grouped: of the first group), and the two candidates' ms per step
 * (candidate_ms: room for 2, may be NULL).  At most 48 runs per batch. */
int mj_mb_tuning(const mj_mb* mb, int* threads, double* candidate_ms);

/* Forces the form of a step (threads = 128 or 256: one kernel of all orders
 * per step; -1: grouped by order, below; -2: unions, below: of the whole
 * batch when it has one order, else of every order group), or 0 to time the
 * forms again at the next advance. */
int mj_mb_set_config(mj_mb* mb, int threads);

/* A batch of several orders also holds one sub-batch per order, each running
 * the kernel instance of its order alone; a step can then be one cooperative
 * launch per order (in increasing order) instead of one launch of the
 * all-orders kernel.  The first advance times this grouped form beside the
 * two configurations of the all-orders kernel (runs restored afterwards) and
 * keeps the fastest.  Within the grouped form each group is timed both ways:
 * its batch kernel, or its runs' own step kernels (those of mj_lf_advance)
 * one run after the other, and keeps the faster (large meshes of high order
 * run well on their own kernels, many small ones batched).  Reports whether
 * the grouped form is in use, the number of order groups (0 for a batch of
 * one order) and its timed ms per step (any output may be NULL).  No
 * reference counterpart. */
int mj_mb_grouping(const mj_mb* mb, int* grouped, int* n_groups, double* grouped_ms);

/* Group `group` (0 .. n_groups-1, in increasing order): its order, runs,
 * 1 when it steps with its runs' own kernels, and the timed ms per step of
 * both forms (any output may be NULL). */
int mj_mb_group_info(const mj_mb* mb, int group, int* order, int* n_runs, int* own_kernels, double* batch_ms,
                     double* own_ms);

/* Union form.  The runs of one order (the whole batch, or an order group)
 * can also step as ONE operator over the disjoint union of their meshes:
 * dofs, elements and incidences concatenated in run order (every dof keeps
 * its elements and its sum order, so results are bitwise those of the runs'
 * own kernels), one autotuned element kernel and one streaming gather over
 * all of them, then one launch applying each run's source with its own pulse,
 * counter and dt.  The batch copies the runs' states into the union at the
 * start of an advance and back at its end; factors changed since
 * (mj_op_set_element_scale) are copied again at the next advance.  The
 * autotuner times it beside the batch kernel (and, in a group, beside the
 * runs' own kernels).  group = -1: the batch itself, else an order group.
 * Reports whether that union steps the runs, its timed ms per step, its
 * element kernel's tile size and its dofs (0 when the runs are too large for
 * one union's int32 indexing and have none).  Any output may be NULL. */
int mj_mb_union_info(const mj_mb* mb, int group, int* in_use, double* union_ms, int* tile_elems, int* n_dof);

/* ---- media update and adjoint ------------------------------------------ */

/* Scales the stiffness factors of every element: factors(e) = scale[e] *
 * factors given at creation (e.g. unit-mu factors scaled by mu_e = c_e^2).
 * Host array of n_elt values >= 0.  The role of changing the media
 * references (MateriauDielec) and recomputing Glob_matMass_Bh
 * (MONTJOIE/src/Elliptic/Helmholtz/VarHelmholtz.cxx:54-131). */
int mj_op_set_element_scale(mj_op* op, const double* scale);

typedef struct mj_adj mj_adj;

/* Discrete adjoint of the many-source leap-frog of `b` over nsteps steps from
 * zero initial conditions, with the forward states checkpointed every
 * checkpoint_every steps (0: ceil(sqrt(nsteps))) and replayed segment by
 * segment in the backward sweep.  checkpoint_every >= nsteps keeps every
 * forward state (nsteps x n_dof x S floats, checked against the free device
 * memory; MJ_ERR_ARG when it does not fit): nothing is recomputed, and the
 * gradient is bit for bit that of any other interval.  No reference
 * counterpart: the reference has no time-domain adjoint.  `b` must have
 * receivers. */
int mj_adj_create(mj_lfb* b, int nsteps, int checkpoint_every, mj_adj** out);

/* The same adjoint with binomial checkpointing (Griewank and Walther's
 * revolve) under a budget of `snapshots` stored forward states (each a pair
 * U^k, U^{k+1}; three more states are working buffers): the schedule that
 * recomputes the fewest forward steps for that budget, planned at creation
 * by dynamic programming (nsteps^2 x snapshots <= 4e8).  The forward sweep
 * stores the schedule's first checkpoints as it passes them.  The gradient
 * is bit for bit that of mj_adj_create: the same adjoint steps run on the
 * same forward states in the same order.  No reference counterpart. */
int mj_adj_create_revolve(mj_lfb* b, int nsteps, int snapshots, mj_adj** out);

/* The binomial schedule of mj_adj_create_revolve, host only (no GPU): the
 * chain of forward states x_k = (U^k, U^{k+1}), k = 1..nsteps-1, visited by
 * the adjoint in the order x_{nsteps-1}, ..., x_1, with x_1 in snapshot slot
 * 0.  actions (room for `capacity` triples, may be NULL) receive (kind, k,
 * slot) with kind 0 = restore slot into the current state x_k, 1 = advance
 * the current state to x_k, 2 = store the current state x_k in slot, 3 =
 * visit x_k; *n_actions their count; *backward_steps the forward steps the
 * whole schedule takes from x_1 (the minimum for that many snapshots). */
int mj_revolve_schedule(int nsteps, int snapshots, int capacity, int* actions, int* n_actions,
                        long long* backward_steps);

/* Schedule facts: 1 for binomial checkpointing (else uniform), stored state
 * pairs, forward steps of one forward + backward pass (nsteps + the steps the
 * backward sweep recomputes) and the checkpoint memory in bytes (any output
 * may be NULL). */
int mj_adj_info(const mj_adj* a, int* revolve, int* snapshots, long long* forward_steps, size_t* device_bytes);
int mj_adj_destroy(mj_adj* a);

/* Forward run storing checkpoints; traces (host, may be NULL) receive the
 * receiver values of U^0..U^nsteps at traces[(k*S + s)*(nsteps+1) + n]. */
int mj_adj_forward(mj_adj* a, double* traces);

/* Backward sweep for the loss J = sum g_n(U^n) whose gradient with respect
 * to the traces is `residual` (same layout as traces, host).  Returns
 * grad[e] = coef[e] * sum_{n=1}^{nsteps-1} sum_s lambda^{n+1}_s^T A_e U^n_s
 * (A_e the element's stiffness as currently scaled), host arrays of n_elt.
 * With A_e = c_e^2 A_e^(1), coef[e] = -2 dt^2 / c_e gives dJ/dc_e.  Each
 * term is evaluated as (A_e lambda^{n+1})^T U^n (A_e is symmetric) inside the
 * adjoint step that computes A_e lambda^{n+1}, in one summation order
 * whatever the step's variant or form and the checkpoint schedule. */
int mj_adj_backward(mj_adj* a, const double* residual, const double* coef, double* grad);

/* ---- setup helpers (geometry, numbering, mass) ------------------------ */

/* Global numbering of a conforming hexahedral mesh of order r: vertices,
 * edges, faces and interiors get shared dofs with consistent orientation
 * (the role of MeshNumbering/NumberMap, MONTJOIE/src/Mesh/NumberMap.cxx).
 * hexes: n_elt x 8 vertex indices in reference-cube order; nodle_out:
 * n_elt x (r+1)^3 in reference local order.  Dofs are numbered in the order
 * elements first touch them, each edge's, face's and element interior's
 * interior nodes as one block when the entity is first met.  *n_dof
 * receives the count. */
int mj_number_hex_mesh(int order, int n_elt, int n_vert, const int32_t* hexes, int32_t* nodle_out,
                       int* n_dof);

/* FP64 geometry on the device: per quadrature point J*w and the stiffness
 * factors B = (J w) DF^-1 mu_e DF^-T of straight-sided (trilinear) hexahedra
 * (VarGeometryProblem.cxx:685-759, VarHelmholtz.cxx:54-131).  verts:
 * n_elt x 8 x 3 host; mu: n_elt host.  factors_out (n_elt x Q x 6) and
 * jw_out (n_elt x Q) are host buffers (either may be NULL); positions_out
 * (n_elt x Q x 3, may be NULL) gets the physical points.  Returns
 * MJ_ERR_GEOMETRY when a Jacobian is not positive. */
int mj_geometry(int order, int n_elt, const double* verts, const double* mu, double* factors_out,
                double* jw_out, double* positions_out);

/* Lumped mass D_i = sum rho_e J w over the points on dof i (TimeAcoustic.cxx:889-965)
 * accumulated on the host in element order (the reference's assembly order,
 * so sums round alike).  rho may be NULL (1). */
int mj_lumped_mass(int order, int n_elt, int n_dof, const int32_t* nodle, const double* jw,
                   const double* rho, double* mass_out);

/* ---- allocation-free product ------------------------------------------ */

/* Largest n_elt*(order+1)^3 accepted by mj_stiffness_mltadd_static. */
#define MJ_STATIC_SCRATCH_POINTS 4194304

/* y <- beta*y + alpha*A*x in FP64 without allocating any memory.
 * No counterpart in the reference: it serves callers that must not let a
 * library allocate GPU memory.  Examples are a solver whose device memory is
 * carved out of one arena owned by another allocator, or a time loop that
 * stages every buffer up front and must not call cudaMalloc/cudaFree later,
 * because those calls can synchronise the device and fragment the arena.
 * All arrays are DEVICE pointers the caller owns, in the reference layout:
 * nodle (n_elt x (r+1)^3 int32), factors (n_elt x (r+1)^3 x 6), x and y
 * (n_dof doubles).  The element-local scratch is a fixed array of
 * MJ_STATIC_SCRATCH_POINTS doubles (32 MiB) inside the library.  Every GPU
 * that loads the library holds it until the process exits.  Larger meshes are
 * rejected with MJ_ERR_ARG.  Every call looks up that array's device address
 * in the current device's context (no allocation); the first call on a device
 * also loads the library's device code there, so make the first call on each
 * device before any stream capture.  All calls share the one array and keep
 * no state in it between calls, so calls that overlap on the GPU (other
 * streams or host threads) race; serialise them.  The work is ordered on
 * `stream` (a cudaStream_t, NULL = legacy default stream) and the call waits
 * for it: it returns once the product is in y.  The scatter uses atomic
 * additions, so the result equals mj_op_mltadd's up to rounding order. */
int mj_stiffness_mltadd_static(int order, int n_elt, int n_dof, const int32_t* nodle, const double* factors,
                               double alpha, const double* x, double beta, double* y, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MONTJOIE_GB300_H */
