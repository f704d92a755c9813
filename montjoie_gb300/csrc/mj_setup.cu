// One-time setup: 1-D Gauss-Lobatto rule, local and global hexahedral
// numbering, FP64 geometry on the device, lumped mass.
#include <cuda_runtime.h>

#include <array>
#include <cmath>
#include <cstring>
#include <vector>

#include "mj_common.cuh"

namespace mj {

namespace {
const int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
const int kEdge[12][2] = {{0, 1}, {1, 2}, {3, 2}, {0, 3}, {0, 4}, {1, 5}, {2, 6}, {3, 7}, {4, 5}, {5, 6}, {7, 6}, {4, 7}};
}  // namespace

std::vector<int> hex_local_numbering(int r) {
  const int n = r + 1;
  std::vector<int> num(n * n * n, -1);
  auto at = [&](int i, int j, int k) -> int& { return num[(i * n + j) * n + k]; };
  int node = 0;
  for (int v = 0; v < 8; v++) at(kCorner[v][0] * r, kCorner[v][1] * r, kCorner[v][2] * r) = node++;
  for (int e = 0; e < 12; e++) {
    const int* a = kCorner[kEdge[e][0]];
    const int* b = kCorner[kEdge[e][1]];
    for (int l = 1; l < r; l++) {
      // point at parameter l from corner a towards corner b
      at(a[0] * r + l * (b[0] - a[0]), a[1] * r + l * (b[1] - a[1]), a[2] * r + l * (b[2] - a[2])) = node++;
    }
  }
  for (int p = 1; p < r; p++) for (int q = 1; q < r; q++) at(0, p, q) = node++;
  for (int p = 1; p < r; p++) for (int q = 1; q < r; q++) at(p, 0, q) = node++;
  for (int p = 1; p < r; p++) for (int q = 1; q < r; q++) at(p, q, 0) = node++;
  for (int p = 1; p < r; p++) for (int q = 1; q < r; q++) at(p, q, r) = node++;
  for (int p = 1; p < r; p++) for (int q = 1; q < r; q++) at(p, r, q) = node++;
  for (int p = 1; p < r; p++) for (int q = 1; q < r; q++) at(r, p, q) = node++;
  for (int p = 1; p < r; p++)
    for (int q = 1; q < r; q++)
      for (int s = 1; s < r; s++) at(p, q, s) = node++;
  return num;
}

// Legendre polynomial P_r and derivative on [-1,1].
static void legendre_pd(int r, double x, double& p, double& dp) {
  double p0 = 1.0, p1 = x, d0 = 0.0, d1 = 1.0;
  if (r == 0) { p = 1.0; dp = 0.0; return; }
  for (int k = 1; k < r; k++) {
    const double p2 = ((2.0 * k + 1.0) * x * p1 - k * p0) / (k + 1.0);
    const double d2 = d0 + (2.0 * k + 1.0) * p1;
    p0 = p1; p1 = p2; d0 = d1; d1 = d2;
  }
  p = p1; dp = d1;
}

void gauss_lobatto(int r, double* pts, double* wts) {
  // Interior nodes: roots of P_r' (Newton on P_r', second derivative from the
  // Legendre equation), weights 1/(r(r+1) P_r(x)^2) on [0,1].
  const double pi = 3.14159265358979323846;
  std::vector<double> x(r + 1);
  for (int i = 0; i <= r; i++) x[i] = -std::cos(pi * i / r);
  for (int i = 1; i < r; i++)
    for (int it = 0; it < 100; it++) {
      double p, dp;
      legendre_pd(r, x[i], p, dp);
      const double d2 = (2.0 * x[i] * dp - r * (r + 1.0) * p) / (1.0 - x[i] * x[i]);
      const double step = dp / d2;
      x[i] -= step;
      if (std::fabs(step) < 1e-17) break;
    }
  for (int i = 0; i <= r; i++) {
    double p, dp;
    legendre_pd(r, x[i], p, dp);
    pts[i] = 0.5 * (x[i] + 1.0);
    wts[i] = 1.0 / (r * (r + 1.0) * p * p);
  }
  pts[0] = 0.0;
  pts[r] = 1.0;
}

void gl_derivative_matrix(int r, const double* pts, double* g) {
  const int n = r + 1;
  std::vector<double> c(n);
  for (int i = 0; i < n; i++) {
    double prod = 1.0;
    for (int j = 0; j < n; j++)
      if (j != i) prod *= pts[i] - pts[j];
    c[i] = 1.0 / prod;
  }
  for (int b = 0; b < n; b++) {
    double sum = 0.0;
    for (int a = 0; a < n; a++)
      if (a != b) {
        g[a * n + b] = c[a] / (c[b] * (pts[b] - pts[a]));
        sum += g[a * n + b];
      }
    g[b * n + b] = -sum;
    if (std::fabs(g[b * n + b]) <= 1e3 * 2.220446049250313e-16) g[b * n + b] = 0.0;
  }
}

// ------------------------------------------------------------ geometry kernel

struct GeomParams {
  int n, Q;
  double pts[kMaxN];
  double wts[kMaxN];
};

__constant__ unsigned char c_coord[kMaxN * kMaxN * kMaxN * 3];  // local index -> (i,j,k)

// Output layout of k_geometry.  Reference layout (Qp = 0): point t = e*Q + q
// in local (NumDofs3D) order, factors fac[6t + c], jw[t], xq[3t + d].
// Element-major layout (Qp > 0, the operators' layout): slot
// p = (k*n + j)*n + i of element e, factors fac[(e*6 + c)*Qp + p] (FP64, or
// FP32 in fac32), jw[e*Qp + p], xq[(e*3 + d)*Qp + p].  Both layouts come from
// the same arithmetic, so every setup path gives the same bits.
struct GeomOut {
  int Qp;
  double* fac;
  float* fac32;
  double* jw;
  double* xq;
};

__global__ void k_geometry(const double* __restrict__ verts, const double* __restrict__ mu, int n_elt,
                           const GeomParams P, const GeomOut out, int* __restrict__ bad) {
  const long long total = (long long)n_elt * P.Q;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int e = (int)(t / P.Q);
    const int q = (int)(t - (long long)e * P.Q);
    const int ci = c_coord[3 * q], cj = c_coord[3 * q + 1], ck = c_coord[3 * q + 2];
    const long long pe = out.Qp ? (long long)e * out.Qp + (ck * P.n + cj) * P.n + ci : t;  // this point's slot
    const double x = P.pts[ci], y = P.pts[cj], z = P.pts[ck];
    const double w = P.wts[ci] * P.wts[cj] * P.wts[ck];
    const double* v = verts + (size_t)e * 24;
    double F[3] = {0, 0, 0}, DF[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    const double cx[2] = {1.0 - x, x}, cy[2] = {1.0 - y, y}, cz[2] = {1.0 - z, z};
    const double dd[2] = {-1.0, 1.0};
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const int a = (c == 1 || c == 2 || c == 5 || c == 6), b = (c == 2 || c == 3 || c == 6 || c == 7), g = (c >= 4);
      const double N = cx[a] * cy[b] * cz[g];
      const double Nx = dd[a] * cy[b] * cz[g], Ny = cx[a] * dd[b] * cz[g], Nz = cx[a] * cy[b] * dd[g];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        const double vc = v[c * 3 + d];
        F[d] += N * vc;
        DF[d][0] += Nx * vc;
        DF[d][1] += Ny * vc;
        DF[d][2] += Nz * vc;
      }
    }
    const double c00 = DF[1][1] * DF[2][2] - DF[1][2] * DF[2][1];
    const double c01 = DF[1][2] * DF[2][0] - DF[1][0] * DF[2][2];
    const double c02 = DF[1][0] * DF[2][1] - DF[1][1] * DF[2][0];
    const double J = DF[0][0] * c00 + DF[0][1] * c01 + DF[0][2] * c02;
    if (!(J > 0.0)) atomicAdd(bad, 1);
    const double iJ = 1.0 / J;
    double inv[3][3];
    inv[0][0] = c00 * iJ;
    inv[1][0] = c01 * iJ;
    inv[2][0] = c02 * iJ;
    inv[0][1] = (DF[0][2] * DF[2][1] - DF[0][1] * DF[2][2]) * iJ;
    inv[1][1] = (DF[0][0] * DF[2][2] - DF[0][2] * DF[2][0]) * iJ;
    inv[2][1] = (DF[0][1] * DF[2][0] - DF[0][0] * DF[2][1]) * iJ;
    inv[0][2] = (DF[0][1] * DF[1][2] - DF[0][2] * DF[1][1]) * iJ;
    inv[1][2] = (DF[0][2] * DF[1][0] - DF[0][0] * DF[1][2]) * iJ;
    inv[2][2] = (DF[0][0] * DF[1][1] - DF[0][1] * DF[1][0]) * iJ;
    const double jwq = J * w;
    if (out.jw) out.jw[pe] = jwq;
    if (out.xq)
#pragma unroll
      for (int d = 0; d < 3; d++) out.xq[out.Qp ? ((long long)e * 3 + d) * out.Qp + (pe - (long long)e * out.Qp)
                                                : 3 * t + d] = F[d];
    if (out.fac || out.fac32) {
      const double s = jwq * mu[e];
      const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
      for (int c = 0; c < 6; c++) {
        const int a = ia[c], b = ib[c];
        const double v = s * (inv[a][0] * inv[b][0] + inv[a][1] * inv[b][1] + inv[a][2] * inv[b][2]);
        const long long fi = out.Qp ? ((long long)e * 6 + c) * out.Qp + (pe - (long long)e * out.Qp) : 6 * t + c;
        if (out.fac) out.fac[fi] = v;
        else out.fac32[fi] = (float)v;
      }
    }
  }
}

// Values of the element-major points scattered to their incidence slots:
// tmp[slot_e[e*Qp + p]] = v(e, p), for the lumped mass (v = rho_e J w) or the
// Gaussian source (v = J w g(|x - c|) inside the ball, 0 outside, with the
// distance rounded as sqrt((dx*dx + dy*dy) + dz*dz), no fused multiply-add).
struct SlotValues {
  int n_elt, Q, Qp, n;
  const double* jw;    // element-major J w
  const double* xq;    // element-major positions (source only)
  const double* rho;   // per element, or NULL (mass)
  const int* slot;
  double cx, cy, cz, R, alpha, beta;
  int gauss;
};

__global__ void k_slot_values(const SlotValues a, double* __restrict__ tmp) {
  const long long total = (long long)a.n_elt * a.Q;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int e = (int)(t / a.Q);
    const int p = (int)(t - (long long)e * a.Q);  // p < Q: a real point of the element (p = (k*n + j)*n + i)
    const long long pe = (long long)e * a.Qp + p;
    double v;
    if (a.gauss) {
      const double dx = a.xq[((long long)e * 3) * a.Qp + p] - a.cx;
      const double dy = a.xq[((long long)e * 3 + 1) * a.Qp + p] - a.cy;
      const double dz = a.xq[((long long)e * 3 + 2) * a.Qp + p] - a.cz;
      const double rr = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
      v = rr < a.R ? __dmul_rn(__dmul_rn(a.jw[pe], a.beta), exp(-a.alpha * __dmul_rn(rr, rr))) : 0.0;
    } else {
      v = a.rho ? __dmul_rn(a.rho[e], a.jw[pe]) : a.jw[pe];
    }
    tmp[a.slot[pe]] = v;
  }
}

// out[d] = 0 + tmp[ptr[d]] + tmp[ptr[d] + 1] + ... (the dof's incidences in
// element order: the order of the reference's element-by-element assembly).
__global__ void k_csr_sum(const double* __restrict__ tmp, const int* __restrict__ ptr, int n_dof,
                          double* __restrict__ out) {
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < n_dof; d += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int q = ptr[d]; q < ptr[d + 1]; q++) s = __dadd_rn(s, tmp[q]);
    out[d] = s;
  }
}

}  // namespace mj

using namespace mj;

namespace {

// Open-addressing table from an entity key (an edge: its two vertices; a
// face: three of its vertices in canonical order) to the offset of the
// entity's interior node ids in a flat pool (ids -1 until numbered).  A key
// starts probing at 16 x its smallest vertex, so the entities of nearby
// vertices (those of consecutive elements) sit together in memory; a regular
// vertex of a hexahedral mesh is the smallest vertex of at most 6 edges and
// 12 faces, so its keys mostly fit its own 16 slots.
struct EntityTable {
  static constexpr int kPerVertex = 16;
  std::vector<uint64_t> khi;
  std::vector<uint32_t> klo;
  std::vector<int64_t> off;  // -1: empty slot
  size_t cap = 0;
  explicit EntityTable(size_t n_vert) : cap(n_vert * kPerVertex + 64) {
    khi.assign(cap, 0);
    klo.assign(cap, 0);
    off.assign(cap, -1);
  }
  // Offset of the key's ids; a new key takes `width` fresh ids (-1) at the end of the pool.
  int64_t find_or_add(uint32_t minv, uint64_t hi, uint32_t lo, std::vector<int>& pool, int width) {
    for (size_t i = (size_t)minv * kPerVertex;; i = (i + 1 == cap) ? 0 : i + 1) {
      if (off[i] < 0) {
        khi[i] = hi;
        klo[i] = lo;
        off[i] = (int64_t)pool.size();
        pool.resize(pool.size() + width, -1);
        return off[i];
      }
      if (khi[i] == hi && klo[i] == lo) return off[i];
    }
  }
};

}  // namespace

extern "C" {

int mj_number_hex_mesh(int order, int n_elt, int n_vert, const int32_t* hexes, int32_t* nodle_out, int* n_dof) {
  MJ_CHECK_ARG(order >= 1 && order <= kMaxOrder, "mj_number_hex_mesh: order must be in [1, 8]");
  MJ_CHECK_ARG(n_elt > 0 && n_vert > 0 && hexes && nodle_out && n_dof, "mj_number_hex_mesh: bad argument");
  const int r = order, n = r + 1, Q = n * n * n, m = r - 1;
  const std::vector<int> num = hex_local_numbering(r);
  for (long long t = 0; t < 8LL * n_elt; t++)
    MJ_CHECK_ARG(hexes[t] >= 0 && hexes[t] < n_vert, "mj_number_hex_mesh: vertex index out of range");
  std::vector<int> vdof(n_vert, -1);
  // edge / face -> offset of its interior node ids (canonical order) in a pool
  EntityTable edges((size_t)n_vert), faces((size_t)n_vert);
  std::vector<int> epool, fpool;
  epool.reserve((size_t)n_elt * 3 * std::max(m, 0) + 16);
  fpool.reserve((size_t)n_elt * 3 * std::max(m * m, 0) + 16);
  int corner_of[2][2][2];
  for (int c = 0; c < 8; c++) corner_of[kCorner[c][0]][kCorner[c][1]][kCorner[c][2]] = c;
  // Every node of the reference element, in the order nodes are numbered:
  // tensor order (i fastest, then j, then k), so consecutive nodes along x
  // of an element mostly get consecutive numbers (coalesced gathers).  kind
  // 0: vertex (corner a); 1: edge along axis a at the other coordinates
  // (b, c) in {0,1}^2, node l along it; 2: face fixed along axis a on side
  // b, node (c, l) on its two varying axes; 3: interior.
  struct NodeDesc { int ql, kind, a, b, c, l; };
  std::vector<NodeDesc> nodes;
  for (int k = 0; k < n; k++)
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        const int cc[3] = {i, j, k};
        // interior: b = (i-1) + m((j-1) + m(k-1)), the node's place in the element's interior block
        NodeDesc nd{num[(i * n + j) * n + k], 3, 0, (i - 1) + (r - 1) * ((j - 1) + (r - 1) * (k - 1)), 0, 0};
        int nb = 0;
        for (int d = 0; d < 3; d++) nb += (cc[d] == 0 || cc[d] == r);
        if (nb == 3) {
          nd.kind = 0;
          nd.a = corner_of[i / r][j / r][k / r];
        } else if (nb == 2) {
          int ax = 0;
          for (int d = 0; d < 3; d++)
            if (cc[d] != 0 && cc[d] != r) ax = d;
          const int o1 = ax == 0 ? 1 : 0, o2 = ax == 2 ? 1 : 2;
          nd = {nd.ql, 1, ax, cc[o1] / r, cc[o2] / r, cc[ax]};
        } else if (nb == 1) {
          int fx = 0;
          for (int d = 0; d < 3; d++)
            if (cc[d] == 0 || cc[d] == r) fx = d;
          const int pa = (fx == 0) ? 1 : 0, qa = (fx == 2) ? 1 : 2;
          nd = {nd.ql, 2, fx, cc[fx] / r, cc[pa], cc[qa]};
        }
        nodes.push_back(nd);
      }
  long long next = 0;
  auto fresh = [&](int& id) {
    if (id < 0) id = (int)next++;
    return id;
  };
  // an edge's or a face's interior nodes take consecutive ids, in their
  // canonical order, when the entity is first met; so does an element's
  // interior (every entity's dofs form one block: the gathers of an
  // element's u touch fewer sectors)
  auto fresh_block = [&](std::vector<int>& pool, int64_t base, int width) {
    if (pool[base] < 0)
      for (int t = 0; t < width; t++) pool[base + t] = (int)next++;
  };
  for (int e = 0; e < n_elt; e++) {
    const int32_t* hv = hexes + 8LL * e;
    auto gvert = [&](int ci, int cj, int ck) { return (int)hv[corner_of[ci][cj][ck]]; };
    // the element's 12 edges (axis, the other two coordinates) and 6 faces
    // (fixed axis, side): pool offset and orientation, one lookup each
    int64_t ebase[3][2][2] = {};
    bool efwd[3][2][2] = {};
    int64_t fbase[3][2] = {};
    int fos[3][2] = {}, foq[3][2] = {};
    bool fswap[3][2] = {};
    if (m > 0) {
      for (int ax = 0; ax < 3; ax++)
        for (int a = 0; a < 2; a++)
          for (int b = 0; b < 2; b++) {
            int lo[3], hi[3];
            const int o1 = ax == 0 ? 1 : 0, o2 = ax == 2 ? 1 : 2;
            lo[o1] = hi[o1] = a;
            lo[o2] = hi[o2] = b;
            lo[ax] = 0;
            hi[ax] = 1;
            const int ga = gvert(lo[0], lo[1], lo[2]), gb = gvert(hi[0], hi[1], hi[2]);
            const uint64_t key = ((uint64_t)(uint32_t)std::min(ga, gb) << 32) | (uint32_t)std::max(ga, gb);
            ebase[ax][a][b] = edges.find_or_add((uint32_t)std::min(ga, gb), key, 0xFFFFFFFFu, epool, m);
            efwd[ax][a][b] = ga < gb;
          }
      for (int fx = 0; fx < 3; fx++)
        for (int side = 0; side < 2; side++) {
          const int pa = (fx == 0) ? 1 : 0, qa = (fx == 2) ? 1 : 2;  // the two varying axes
          auto corner = [&](int sp, int sq) {
            int cc[3];
            cc[fx] = side;
            cc[pa] = sp;
            cc[qa] = sq;
            return gvert(cc[0], cc[1], cc[2]);
          };
          const int g[2][2] = {{corner(0, 0), corner(0, 1)}, {corner(1, 0), corner(1, 1)}};
          // canonical frame: origin = smallest vertex; first axis towards its
          // smaller neighbour.
          int os = 0, oq = 0;
          for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++)
              if (g[a][b] < g[os][oq]) { os = a; oq = b; }
          const int nP = g[1 - os][oq], nQ = g[os][1 - oq];
          const bool swap = nQ < nP;  // first canonical axis is q
          const uint64_t hi = ((uint64_t)(uint32_t)g[os][oq] << 32) | (uint32_t)(swap ? nQ : nP);
          fbase[fx][side] = faces.find_or_add((uint32_t)g[os][oq], hi, (uint32_t)(swap ? nP : nQ), fpool, m * m);
          fos[fx][side] = os;
          foq[fx][side] = oq;
          fswap[fx][side] = swap;
        }
    }
    int32_t* out = nodle_out + (size_t)e * Q;
    long long ibase = -1;  // first id of this element's interior block
    for (const NodeDesc& nd : nodes) {
      int dof;
      switch (nd.kind) {
        case 0: dof = fresh(vdof[hv[nd.a]]); break;
        case 1: {
          const int64_t base = ebase[nd.a][nd.b][nd.c];
          fresh_block(epool, base, m);
          dof = epool[base + (efwd[nd.a][nd.b][nd.c] ? nd.l : r - nd.l) - 1];
          break;
        }
        case 2: {
          int p = nd.c, q = nd.l;
          if (fos[nd.a][nd.b]) p = r - p;
          if (foq[nd.a][nd.b]) q = r - q;
          const int u = fswap[nd.a][nd.b] ? q : p, v = fswap[nd.a][nd.b] ? p : q;
          const int64_t base = fbase[nd.a][nd.b];
          fresh_block(fpool, base, m * m);
          dof = fpool[base + (u - 1) * m + (v - 1)];
          break;
        }
        default: {  // interior node: its place nd.b in the element's interior block
          if (ibase < 0) {
            ibase = next;
            next += (long long)m * m * m;
          }
          dof = (int)(ibase + nd.b);
        }
      }
      if (next > INT32_MAX) {
        set_error("mj_number_hex_mesh: too many dofs for int32");
        return MJ_ERR_ARG;
      }
      out[nd.ql] = dof;
    }
  }
  *n_dof = (int)next;
  return MJ_OK;
}

int mj_geometry(int order, int n_elt, const double* verts, const double* mu, double* factors_out, double* jw_out,
                double* positions_out) {
  MJ_CHECK_ARG(order >= 1 && order <= kMaxOrder, "mj_geometry: order must be in [1, 8]");
  MJ_CHECK_ARG(n_elt > 0 && verts, "mj_geometry: bad argument");
  MJ_CHECK_ARG(!factors_out || mu, "mj_geometry: factors need mu");
  const int r = order, n = r + 1, Q = n * n * n;
  GeomParams P{};
  P.n = n;
  P.Q = Q;
  gauss_lobatto(r, P.pts, P.wts);
  const std::vector<int> num = hex_local_numbering(r);
  std::vector<unsigned char> coord(Q * 3);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      for (int k = 0; k < n; k++) {
        const int q = num[(i * n + j) * n + k];
        coord[3 * q] = (unsigned char)i;
        coord[3 * q + 1] = (unsigned char)j;
        coord[3 * q + 2] = (unsigned char)k;
      }
  MJ_CUDA(cudaMemcpyToSymbol(c_coord, coord.data(), coord.size()));
  const size_t pts = (size_t)n_elt * Q;
  DevBuf dv, dmu, dfac, djw, dxq, dbad;
  MJ_CUDA(dv.alloc(sizeof(double) * 24 * n_elt));
  MJ_CUDA(cudaMemcpy(dv.ptr, verts, sizeof(double) * 24 * n_elt, cudaMemcpyHostToDevice));
  if (factors_out) {
    MJ_CUDA(dmu.alloc(sizeof(double) * n_elt));
    MJ_CUDA(cudaMemcpy(dmu.ptr, mu, sizeof(double) * n_elt, cudaMemcpyHostToDevice));
    MJ_CUDA(dfac.alloc(sizeof(double) * 6 * pts));
  }
  if (jw_out) MJ_CUDA(djw.alloc(sizeof(double) * pts));
  if (positions_out) MJ_CUDA(dxq.alloc(sizeof(double) * 3 * pts));
  MJ_CUDA(dbad.alloc(sizeof(int)));
  MJ_CUDA(cudaMemset(dbad.ptr, 0, sizeof(int)));
  const int blocks = (int)std::min<size_t>((pts + 255) / 256, (size_t)sm_count() * 32);
  const GeomOut go{0, dfac.as<double>(), nullptr, djw.as<double>(), dxq.as<double>()};
  k_geometry<<<blocks, 256>>>(dv.as<double>(), dmu.as<double>(), n_elt, P, go, dbad.as<int>());
  count_launch();
  MJ_CUDA(cudaGetLastError());
  int bad = 0;
  MJ_CUDA(cudaMemcpy(&bad, dbad.ptr, sizeof(int), cudaMemcpyDeviceToHost));
  if (factors_out) MJ_CUDA(cudaMemcpy(factors_out, dfac.ptr, sizeof(double) * 6 * pts, cudaMemcpyDeviceToHost));
  if (jw_out) MJ_CUDA(cudaMemcpy(jw_out, djw.ptr, sizeof(double) * pts, cudaMemcpyDeviceToHost));
  if (positions_out) MJ_CUDA(cudaMemcpy(positions_out, dxq.ptr, sizeof(double) * 3 * pts, cudaMemcpyDeviceToHost));
  if (bad) {
    set_error("mj_geometry: " + std::to_string(bad) + " quadrature points with non-positive Jacobian");
    return MJ_ERR_GEOMETRY;
  }
  return MJ_OK;
}

}  // extern "C"

namespace mj {

namespace {
int geom_params(int order, GeomParams* P) {
  const int r = order, n = r + 1;
  *P = GeomParams{};
  P->n = n;
  P->Q = n * n * n;
  gauss_lobatto(r, P->pts, P->wts);
  const std::vector<int> num = hex_local_numbering(r);
  std::vector<unsigned char> coord(P->Q * 3);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      for (int k = 0; k < n; k++) {
        const int q = num[(i * n + j) * n + k];
        coord[3 * q] = (unsigned char)i;
        coord[3 * q + 1] = (unsigned char)j;
        coord[3 * q + 2] = (unsigned char)k;
      }
  MJ_CUDA(cudaMemcpyToSymbol(c_coord, coord.data(), coord.size()));
  return MJ_OK;
}
}  // namespace

int geometry_elem_major(int order, int n_elt, int Qp, const double* verts, const double* mu, double* fac64,
                        float* fac32, double* jw, double* xq, int* bad, cudaStream_t s) {
  GeomParams P;
  int rc = geom_params(order, &P);
  if (rc) return rc;
  const size_t pts = (size_t)n_elt * P.Q;
  const int blocks = (int)std::min<size_t>((pts + 255) / 256, (size_t)sm_count() * 32);
  const GeomOut go{Qp, fac64, fac32, jw, xq};
  k_geometry<<<blocks, 256, 0, s>>>(verts, mu, n_elt, P, go, bad);
  count_launch();
  MJ_CUDA(cudaGetLastError());
  return MJ_OK;
}

int assemble_points(int order, int n_elt, int Qp, const double* jw, const double* xq, const double* rho,
                    const int* slot, const int* ptr, int n_dof, const double* center, double radius, double* tmp,
                    double* out, cudaStream_t s) {
  SlotValues a{};
  a.n_elt = n_elt;
  a.n = order + 1;
  a.Q = a.n * a.n * a.n;
  a.Qp = Qp;
  a.jw = jw;
  a.xq = xq;
  a.rho = rho;
  a.slot = slot;
  a.gauss = center != nullptr;
  if (a.gauss) {
    // g(x) = beta exp(-alpha r^2) for r < R, alpha = -ln(1e-6)/R^2, beta = sqrt(alpha/pi)
    // (GaussianSource::GetAmplitude, MONTJOIE/src/Source/SourceSpatiale.cxx:78-90)
    a.cx = center[0];
    a.cy = center[1];
    a.cz = center[2];
    a.R = radius;
    a.alpha = -std::log(1e-6) / (radius * radius);
    a.beta = std::sqrt(a.alpha / M_PI);
  }
  const size_t pts = (size_t)n_elt * a.Q;
  const int blocks = (int)std::min<size_t>((pts + 255) / 256, (size_t)sm_count() * 32);
  k_slot_values<<<blocks, 256, 0, s>>>(a, tmp);
  k_csr_sum<<<(int)std::min<size_t>(((size_t)n_dof + 255) / 256, (size_t)sm_count() * 32), 256, 0, s>>>(tmp, ptr,
                                                                                                       n_dof, out);
  count_launch(2);
  MJ_CUDA(cudaGetLastError());
  return MJ_OK;
}

}  // namespace mj

extern "C" {

int mj_lumped_mass(int order, int n_elt, int n_dof, const int32_t* nodle, const double* jw, const double* rho,
                   double* mass_out) {
  MJ_CHECK_ARG(order >= 1 && order <= kMaxOrder, "mj_lumped_mass: order must be in [1, 8]");
  MJ_CHECK_ARG(n_elt > 0 && n_dof > 0 && nodle && jw && mass_out, "mj_lumped_mass: bad argument");
  const int Q = (order + 1) * (order + 1) * (order + 1);
  // Element-loop accumulation in the reference's order (AddMatrixWithBC over
  // elements, then points), so sums round identically.
  std::memset(mass_out, 0, sizeof(double) * n_dof);
  for (int e = 0; e < n_elt; e++) {
    const double re = rho ? rho[e] : 1.0;
    for (int q = 0; q < Q; q++) {
      const int d = nodle[(size_t)e * Q + q];
      MJ_CHECK_ARG(d >= 0 && d < n_dof, "mj_lumped_mass: Nodle entry out of range");
      mass_out[d] += re * jw[(size_t)e * Q + q];
    }
  }
  return MJ_OK;
}

}  // extern "C"
