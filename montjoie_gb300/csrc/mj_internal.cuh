// Internal state of an operator, shared by the translation units of the
// library (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <vector>

#include "mj_common.cuh"

struct mj_op {
  int order = 0, n = 0, Q = 0, Qp = 0;
  int n_elt = 0, n_elt_pad = 0, n_dof = 0, precision = MJ_FP64;
  int E = 1, n_tiles = 0, grid_k1 = 1;  // tile size and grid of the element kernel (autotuned)
  bool vec = false;                     // work layout of the element kernel (autotuned)
  bool warp = false;                    // warp-per-element layout (FP32, order 4; autotuned)
  bool packed = false;                  // that layout with packed connectivity (nodle_pk; autotuned)
  bool fs = false;                      // compact layout with one factor stage (FP32; autotuned)
  size_t r_len = 0;                     // element-major slots (n_elt_pad * Qp)
  size_t n_inc = 0;                     // incidences (n_elt * Q); R has n_inc + 1 entries
  mj::DevBuf nodle_e, fac_e, slot_e, R, ptr;
  mj::DevBuf nodle_pk;                  // packed connectivity: dof | rank << 27 (FP32 order 4), or empty
  mj::DevBuf err;                       // device error flag (bounded-wait timeouts)
  mj::DevBuf fac_orig;                  // factors before mj_op_set_element_scale (kept on first use)
  int fac_version = 0;                  // bumped whenever fac_e changes after creation
  mj::DevBuf verts;                     // n_elt x 8 x 3 vertices (operators built from geometry)
  std::vector<int> h_ptr;               // CSR of incidences per dof (host copy)
  double gradphi[mj::kMaxN * mj::kMaxN];
  mj::DevBuf xbuf, ybuf;                // staging for host-vector MltAdd
  cudaStream_t stream = nullptr;
  std::vector<double> tune_ms;          // autotuner timings of the candidates (diagnostic)
  std::vector<int> tune_E, tune_vec;
  size_t device_bytes() const {
    return nodle_e.bytes + fac_e.bytes + fac_orig.bytes + slot_e.bytes + R.bytes + ptr.bytes + xbuf.bytes +
           ybuf.bytes + verts.bytes + nodle_pk.bytes;
  }
};

// State of one leap-frog run (mj_lf_*), shared with the mesh-batch unit.
struct mj_lf {
  mj_op* op = nullptr;
  double dt = 0;
  int n_dof = 0;
  mj::DevBuf src_idx, src_val;  // sparse source (value in op precision)
  mj::DevBuf mass, minv;     // op precision (FP64: D and 1/D; FP32: unused / dt^2/D)
  mj::DevBuf inv_mass64;     // FP64 1/D for the initial step
  mj::DevBuf norm_w;         // FP64 weights, or empty
  mj::DevBuf norm_w32;       // the same rounded to FP32 (FP32 integrators), or empty
  bool norm_is_mass = false; // FP32: the norm weights equal the mass, so the streaming gather's fused norm takes
                             // them as dt^2 / (dt^2/D), from the dt^2/D it stages anyway
  mj::DevBuf rec_idx, rec_w; // receivers
  mj::DevBuf ua, ub;         // state: U^n (cur) and U^{n+1} (next)
  mj::DevBuf du0, tmp;       // staging
  mj::DevBuf partial, norms_d, traces_d, flag;
  mj::DevBuf diag_done, diag_where;  // fused diagnostics: finished-block counter, DiagDev of graph replays
  mj::DevBuf stream_partial;         // per-CTA norm partials of the streaming gather's diagnostics
  mj::DevBuf pulse_d, ctr;   // pulse of every step and the two step counters
  int n_pulse = 0;
  cudaGraphExec_t graph = nullptr, graph_prof = nullptr;
  cudaGraphExec_t graph_diag = nullptr;  // steps with norm and receivers, columns read from diag_where
  bool use_graph = true;  // replay captured steps when no diagnostics are asked
  int n_src = 0, n_rec = 0, n_rec_w = 0;
  double norm_max = 1e30;  // largest |norm| accepted (NormeMaxSolution; the reference's default)
  int step = 0;
  bool initialised = false;
  bool cur_is_a = true;
  cudaStream_t stream = nullptr;
  int norm_blocks = 0;
  // optional per-kernel timing (CUDA events around the two kernels of a step)
  bool profile = false;
  std::vector<cudaEvent_t> ev;
  int ev_used = 0;
  double prof_elem_ms = 0.0, prof_update_ms = 0.0;
  int prof_steps = 0;
  // order-4 modified-equation scheme (mj_lf_set_scheme): second derivative
  // of the pulse, scratch vectors, sources looked up per dof
  int time_order = 2;
  mj::DevBuf pulse3_d;
  int n_pulse3 = 0;
  mj::DevBuf w4, z4, d3_4;
  mj::DevBuf src_mask, src_sidx, src_sval;
  int n_src_sorted = 0;
  // FP32 order-2 step: streaming gather (k_gather_leapfrog_stream) over dof chunks
  bool stream_gather = false;
  mj::DevBuf stream_chunks;
  int n_stream_chunks = 0, stream_grid_ = 0;
  ~mj_lf() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    if (graph) cudaGraphExecDestroy(graph);
    if (graph_prof) cudaGraphExecDestroy(graph_prof);
    if (graph_diag) cudaGraphExecDestroy(graph_diag);
  }
  void* cur() { return cur_is_a ? ua.ptr : ub.ptr; }
  void* next() { return cur_is_a ? ub.ptr : ua.ptr; }
};

// State of S leap-frog runs sharing one mesh (mj_lfb_*), shared by the
// many-source units.
struct mj_lfb {
  mj_op* op = nullptr;
  int S = 0, n_dof = 0;
  double dt = 0;
  int E = 1, L = 32, grid = 1, n_tiles = 0;  // tuned element-kernel variant
  mj::DevBuf R;                                  // element-local results [slot][S]
  mj::DevBuf src_idx, src_val, src_rhs, m, inv_mass64, pulse, ctr;
  int n_src = 0;
  mj::DevBuf ua, ub, stage, rec_idx, rec_w, traces_d;
  int n_pulse = 0, n_rec = 0, n_rec_w = 0;
  int step = 0;
  bool cur_is_a = true, initialised = false;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  std::vector<double> tune_ms;
  // one cooperative kernel per step (mj_rhs_step.cu): chosen variant, launch
  // shape, dof chunks, sources grouped by dof, barrier state, graphs by parity
  bool fused = true;
  int rs_variant = -1, rs_grid = 0, rs_threads = 0, rs_n_chunks = 0;
  mj::DevBuf rs_chunks, rs_src_dof, rs_src_ptr, rs_src_rhs, rs_src_val, rs_sync, rs_err;
  int rs_n_src_dof = 0;
  int rs_en_variant = -1, rs_en_grid = 0;  // the step's EN form (adjoint gradient term): for which variant, its grid
  cudaGraphExec_t rs_graph[2] = {nullptr, nullptr};
  std::vector<double> rs_tune_ms;
  std::vector<int> rs_tune_variant;
  bool rs_profile = false;  // plain launches with per-CTA phase time stamps
  mj::DevBuf rs_stamps;
  ~mj_lfb() {
    if (graph) cudaGraphExecDestroy(graph);
    for (auto& g : rs_graph)
      if (g) cudaGraphExecDestroy(g);
  }
  float* cur() { return (cur_is_a ? ua : ub).as<float>(); }
  float* next() { return (cur_is_a ? ub : ua).as<float>(); }
};

namespace mj {

// Tile sizes E (elements per CTA) instantiated for order n = r + 1, all
// dividing kElemPad (240).
std::vector<int> k1_tile_candidates(int n);

// Element-kernel entry points, one set per precision (mj_k1_f64.cu, mj_k1_f32.cu).
// set_gmat: writes the derivative matrix of order n into that unit's constant memory.
// prepare: sets the shared-memory attribute of variant (n, E) and returns its
//   occupancy (CTAs per SM); fails when the variant does not fit.
// launch: one launch of variant (n, E) on `grid` CTAs.
int k1_set_gmat_f64(int n, const double* g);
int k1_set_gmat_f32(int n, const double* g);
// vec: the vector-line work layout (FP32 only; FP64 uses the compact one).
int k1_prepare_f64(int n, int E, bool vec, int* ctas_per_sm);
int k1_prepare_f32(int n, int E, bool vec, int* ctas_per_sm);
void k1_launch_f64(int n, int E, bool vec, int grid, const void* x, const int* nodle_e, const void* fac_e, void* R,
                   const int* slot_e, int n_tiles, int* err, cudaStream_t s);
void k1_launch_f32(int n, int E, bool vec, int grid, const void* x, const int* nodle_e, const void* fac_e, void* R,
                   const int* slot_e, int n_tiles, int* err, cudaStream_t s);
// Warp-per-element layout (FP32; orders with (r+1)^2 <= 32 that are instantiated).
// packed: the variant reading the packed connectivity (nodle_e = nodle_pk,
// slot_e = the CSR offsets ptr; see kPkDofBits).
std::vector<int> k1_warp_tile_candidates(int n);
// Compact layout with one factor stage (FP32, mj_k1_fs.cu): the same tile
// sizes as the compact layout (k1_tile_candidates).
int k1_set_gmat_fs(int n, const double* g);  // called by k1_set_gmat_f32
int k1_prepare_fs_f32(int n, int E, int* ctas_per_sm);
void k1_launch_fs_f32(int n, int E, int grid, const void* x, const int* nodle_e, const void* fac_e, void* R,
                      const int* slot_e, int n_tiles, int* err, cudaStream_t s);
int k1_prepare_w_f32(int n, int E, bool packed, int* ctas_per_sm);
void k1_launch_w_f32(int n, int E, bool packed, int grid, const void* x, const int* nodle_e, const void* fac_e,
                     void* R, const int* slot_e, int n_tiles, int* err, cudaStream_t s);

// Test instances of two variants compiled with a bulk-copy wait limit of 0
// (the test hook of mj_debug_set_wait_limits): FP32 one element per warp with
// n = 5, E = 2, and FP64 compact with n = 5, E = 4.  Return false (nothing
// launched) for any other variant.
bool k1_launch_w_f32_waits_out(int n, int E, int grid, const void* x, const int* nodle_e, const void* fac_e,
                               void* R, const int* slot_e, int n_tiles, int* err, cudaStream_t s);
bool k1_launch_f64_waits_out(int n, int E, int grid, const void* x, const int* nodle_e, const void* fac_e,
                             void* R, const int* slot_e, int n_tiles, int* err, cudaStream_t s);

// Many right-hand sides (FP32 only, mj_batch.cu).
struct RhsVariant {
  int E, L;
};
std::vector<RhsVariant> k1_rhs_candidates(int n);
int k1_set_gmat_rhs(int n, const double* g);

int stream_grid(int n);

// Setup on the device (mj_setup.cu).  geometry_elem_major: FP64 J w, stiffness
// factors B = (J w) DF^-1 mu DF^-T and positions of every quadrature point of
// straight-sided hexahedra (verts: device n_elt x 8 x 3, mu: device n_elt) in
// the element-major layout of the operators (outputs may be NULL; factors in
// FP64 or FP32); *bad (device) counts non-positive Jacobians.
// assemble_points: out[d] = sum over the dof's incidences, in element order,
// of rho_e J w (center == NULL: lumped mass, rho NULL = 1) or of J w g(x)
// (the Gaussian source of `center` and `radius`); tmp: n_inc doubles.
int geometry_elem_major(int order, int n_elt, int Qp, const double* verts, const double* mu, double* fac64,
                        float* fac32, double* jw, double* xq, int* bad, cudaStream_t s);
int assemble_points(int order, int n_elt, int Qp, const double* jw, const double* xq, const double* rho,
                    const int* slot, const int* ptr, int n_dof, const double* center, double radius, double* tmp,
                    double* out, cudaStream_t s);

// One cooperative kernel per step for S right-hand sides (mj_rhs_step.cu):
// variant choice at creation, and the advance used by mj_lfb_advance.
int lfb_fused_setup(mj_lfb* b);
int lfb_fused_advance(mj_lfb* b, int nsteps, double* traces, int trace_stride, bool use_graph);
void lfb_receivers(mj_lfb* b, const float* u, int stride, int col, cudaStream_t s);
int lfb_phase_ms(const mj_lfb* b, double* out);
int lfb_fused_step_on(mj_lfb* b, float* u0, float* u1, float* out, bool sources, cudaStream_t s);
int lfb_fused_step(mj_lfb* b, cudaStream_t s, float* copy = nullptr);
int lfb_fused_step_en(mj_lfb* b, float* u0, float* u1, float* out, const float* ue, double* gacc,
                      const double* gcoef, cudaStream_t s, bool* done);
int lfb_fused_check(mj_lfb* b, cudaStream_t s);
int lfb_set_step_variant(mj_lfb* b, int E, int LB, int V);

// One time step of a run with its own kernels (the ones mj_lf_advance
// launches), on the given buffers (cur = U^n, overwritten by U^{n+2}; next =
// U^{n+1}) and pulse-counter parity qc, on stream s (capturable).
int lf_step_on(mj_lf* lf, void* cur, const void* next, int qc, cudaStream_t s);

// The union of several FP32 order-2 runs of one order (mesh batch,
// mj_multi.cu): one operator over the disjoint union of their meshes (dofs,
// elements and incidences concatenated in run order, so every dof keeps its
// elements and its sum order) with a tuned element kernel, and an integrator
// state over the union's dofs (dt^2/D and 1/D of each run at its offset, no
// sources: the batch applies each run's own).  dof_off/elt_off: each run's
// first dof and element in the union.  union_copy_factors: the factors of run
// operator op into the union at element elt_off (after a change of op's).
int lf_union_create(const std::vector<mj_lf*>& runs, std::unique_ptr<mj_op>* uop, std::unique_ptr<mj_lf>* ulf,
                    std::vector<int>* dof_off, std::vector<int>* elt_off);
int union_copy_factors(mj_op* uop, const mj_op* op, int elt_off, cudaStream_t s);

// Single-order instances of the many-mesh batch kernel (mj_multi_one.cu):
// the kernel for `threads` per CTA and order n (2..9), and the FP32
// derivative matrix of order n in that translation unit's constant bank.
const void* mb_one_order_kernel(int threads, int n);
int mb_one_order_set_gmat(int n, const float* v);

}  // namespace mj
