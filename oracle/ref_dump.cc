// Test infrastructure only (part of the oracle, never linked into the product).
//
// Driver around the reference's OWN acoustic solver, compiled from the Montjoie
// sources where they lie (see oracle/Makefile).  It runs the unmodified
// reference driver `VarInstationary_Base::RunAll`
// (MONTJOIE/src/Instationary/VarInstationary.cxx:1629-1818) on a deck, and
// hooks the virtual `VirtualOdeSystem::GiveIterate`
// (MONTJOIE/src/Instationary/TimeSchemes.hxx:44) to record, from the
// reference's own objects:
//   - the element->dof connectivity `Nodle` (NumberMap, reference local order),
//   - the stiffness factors Glob_matMass_Bh (VarHelmholtz.cxx:95-123),
//     expanded to one symmetric 3x3 per quadrature point,
//   - Glob_jacobian (J*w per point, VarGeometryProblem.cxx:706-709),
//   - the lumped mass D and its inverse (TimeAcoustic.cxx:889-1000),
//   - the sparse source vector F (VarInstationary.cxx:620-676),
//   - the pulse p(t+dt) of every step and its second derivative
//     (TimeSource.cxx:778-880),
//   - y = beta*y0 + alpha*Kh*x for a caller-given x (FemMatrixFreeClass.cxx:953),
//   - the "Norme solution" of every iterate (VarInstationary.cxx:2696-2745),
//   - selected iterates u^n.
// Everything is written as raw little-endian arrays into an output folder.
//
// Usage: ref_dump deck.ini outdir [--x x.f64 --y0 y0.f64 --alpha a --beta b]
//                                [--snaps 0,10,200] [--no-norms]

#define MONTJOIE_WITH_TWO_DIM
#define MONTJOIE_WITH_THREE_DIM
#define MONTJOIE_WITH_NODAL_H1
#define MONTJOIE_WITH_NODAL_DG
#define SELDON_WITH_PRECONDITIONING
#define MONTJOIE_WITH_TIME_REVERSAL

#include "Hyperbolic/Acoustic/MontjoieAcoustic.hxx"
#include "Elliptic/Helmholtz/ProdMatVectHelmholtz.cxx"
#include "Computation/ProdMatVectScalarH1.cxx"

#include <chrono>
#include <cstdio>
#include <fstream>
#include <set>
#include <sstream>

using namespace Montjoie;

// The Amos Bessel / Lambert-W Fortran routines are off the acoustic path and
// no Fortran compiler is available: link stubs that abort if ever reached.
extern "C" {
void cbesj_(const void*, const double*, int*, int*, void*, int*, int*) { abort(); }
void cbesy_(const void*, const double*, int*, int*, void*, int*, void*, int*) { abort(); }
void cbesk_(const void*, const double*, int*, int*, void*, int*, int*) { abort(); }
void lambert_(const double*, double*) { abort(); }
}

namespace {

template <class T>
void write_raw(const std::string& path, const T* data, size_t n) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) { fprintf(stderr, "cannot write %s\n", path.c_str()); exit(2); }
  fwrite(data, sizeof(T), n, f);
  fclose(f);
}

std::vector<double> read_f64(const std::string& path) {
  std::ifstream in(path, std::ios::binary | std::ios::ate);
  if (!in) { fprintf(stderr, "cannot read %s\n", path.c_str()); exit(2); }
  size_t bytes = in.tellg();
  in.seekg(0);
  std::vector<double> v(bytes / sizeof(double));
  in.read(reinterpret_cast<char*>(v.data()), bytes);
  return v;
}

}  // namespace

class DumpingProblem : public HyperbolicProblem<AcousticEquation<Dimension3> > {
 public:
  std::string outdir;
  std::string xfile, y0file;
  double alpha = 1.0, beta = 0.0;
  std::set<int> snaps;
  bool record_norms = true;
  bool dumped = false;
  std::vector<double> norms, times;
  std::chrono::steady_clock::time_point loop_start;
  double loop_seconds = 0.0;
  int last_n = -1;

  void DumpStatic() {
    auto& pb = this->var_harmonic;
    const int ne = pb.mesh.GetNbElt();
    const int ndof = pb.GetNbDof();
    const ElementReference_Dim<Dimension3>& Fb0 = pb.GetReferenceElement(0);
    const int r = Fb0.GetOrder();
    const int n1 = r + 1;
    const int Q = Fb0.GetNbPointsQuadratureInside();

    // 1-D Gauss-Lobatto rule and derivative matrix, built exactly as the
    // reference element builds them (HexahedronGauss.cxx:263).
    Globatto<Real_wp> lob;
    lob.ConstructQuadrature(r, lob.QUADRATURE_LOBATTO);
    lob.ComputeGradPhi(1e3 * epsilon_machine);
    std::vector<double> pts(n1), wts(n1), grad(n1 * n1);
    for (int i = 0; i < n1; i++) { pts[i] = lob.Points(i); wts[i] = lob.Weights(i); }
    for (int a = 0; a < n1; a++)
      for (int b = 0; b < n1; b++) grad[a * n1 + b] = lob.GradPhi(a, b);
    write_raw(outdir + "/points1d.f64", pts.data(), pts.size());
    write_raw(outdir + "/weights1d.f64", wts.data(), wts.size());
    write_raw(outdir + "/gradphi.f64", grad.data(), grad.size());

    Array3D<int> num3d; Matrix<int> coor;
    MeshNumbering<Dimension3>::ConstructHexahedralNumbering(r, num3d, coor);
    std::vector<int> num(n1 * n1 * n1);
    for (int i = 0; i < n1; i++)
      for (int j = 0; j < n1; j++)
        for (int k = 0; k < n1; k++) num[(i * n1 + j) * n1 + k] = num3d(i, j, k);
    write_raw(outdir + "/numdofs3d.i32", num.data(), num.size());

    std::vector<int> nodle((size_t)ne * Q), eref(ne), affine(ne), variable(ne);
    std::vector<double> verts((size_t)ne * 24), bh((size_t)ne * Q * 6), jw((size_t)ne * Q);
    for (int e = 0; e < ne; e++) {
      const ElementReference_Dim<Dimension3>& Fb = pb.GetReferenceElement(e);
      IVect nod = pb.GetDofNumberOnElement(e);
      for (int j = 0; j < Q; j++) nodle[(size_t)e * Q + j] = nod(j);
      VectR3 s;
      pb.mesh.GetVerticesElement(e, s);
      for (int v = 0; v < 8; v++)
        for (int d = 0; d < 3; d++) verts[(size_t)e * 24 + v * 3 + d] = s(v)(d);
      eref[e] = pb.mesh.Element(e).GetReference();
      affine[e] = pb.mesh.IsElementAffine(e) ? 1 : 0;
      variable[e] = pb.UseNumericalIntegration(e) ? 1 : 0;
      const int nb = pb.Glob_matMass_Bh(e).GetM();
      for (int j = 0; j < Q; j++) {
        // Constant factors (affine, uniform media) are stored once and
        // multiplied by the quadrature weight inside the product
        // (ProdMatVectScalarH1.cxx:447-466); expand them per point here.
        double scale = (nb == 1) ? Fb.WeightsND(j) : 1.0;
        const auto& m = pb.Glob_matMass_Bh(e)(nb == 1 ? 0 : j);
        double* o = &bh[((size_t)e * Q + j) * 6];
        o[0] = scale * m(0, 0); o[1] = scale * m(0, 1); o[2] = scale * m(0, 2);
        o[3] = scale * m(1, 1); o[4] = scale * m(1, 2); o[5] = scale * m(2, 2);
        const int nj = pb.Glob_jacobian(e).GetM();
        jw[(size_t)e * Q + j] = (nj == 1) ? pb.Glob_jacobian(e)(0) * Fb.WeightsND(j)
                                          : pb.Glob_jacobian(e)(j);
      }
    }
    write_raw(outdir + "/nodle.i32", nodle.data(), nodle.size());
    write_raw(outdir + "/verts.f64", verts.data(), verts.size());
    write_raw(outdir + "/elem_ref.i32", eref.data(), eref.size());
    write_raw(outdir + "/affine.i32", affine.data(), affine.size());
    write_raw(outdir + "/variable.i32", variable.data(), variable.size());
    write_raw(outdir + "/bh.f64", bh.data(), bh.size());
    write_raw(outdir + "/jw.f64", jw.data(), jw.size());

    // Lumped mass D (ApplyOperatorDh) and the inverse the scheme uses
    // (SolveOperatorDhPlusdtSh, VarInstationaryInline.cxx:220-224).
    VectReal_wp ones(ndof), D(ndof), invD(ndof);
    ones.Fill(1.0); D.Fill(0.0);
    this->ApplyOperatorDh(Real_wp(1), Real_wp(0), ones, Real_wp(0), D);
    invD.Fill(1.0);
    this->SolveOperatorDhPlusdtSh(invD);
    write_raw(outdir + "/massD.f64", D.GetData(), ndof);
    write_raw(outdir + "/invD.f64", invD.GetData(), ndof);

    // Sparse spatial source F.
    const auto& F = this->sparse_vector_source;
    std::vector<int> fidx(F.GetM());
    std::vector<double> fval(F.GetM());
    for (int i = 0; i < F.GetM(); i++) { fidx[i] = F.Index(i); fval[i] = F.Value(i); }
    write_raw(outdir + "/src_idx.i32", fidx.data(), fidx.size());
    write_raw(outdir + "/src_val.f64", fval.data(), fval.size());

    // Pulse p(t_n + dt) with the reference's own interpolated Ricker, on a
    // private TimeSourceHyperbolic so the solver's window state is untouched.
    const double dt = this->deltat, t0 = this->initial_time, tf = this->final_time;
    const int nsteps = toInteger(ceil(abs(tf - t0) / dt));
    {
      TimeSourceHyperbolic ts;
      VirtualTimeSource<Real_wp>* fsrc = this->GetNewTimeSource();
      ts.Init(fsrc, pb.GetFrequency(), this->epsilon_time, t0);
      std::vector<double> pulse(nsteps);
      for (int n = 0; n < nsteps; n++) {
        double t = t0 + n * dt + dt;
        Real_wp p = 0;
        ts.EvaluateDerivative(t, 1, p);
        pulse[n] = (t >= this->tlimit_source) ? 0.0 : p;
      }
      write_raw(outdir + "/pulse.f64", pulse.data(), pulse.size());
    }
    {
      // d^2 p / dt^2 at the same times (derivative order 3 of the primitive),
      // which the order-4 modified-equation step adds as dt^2 p'' F
      // (ModifiedEquation.cxx:381-385)
      TimeSourceHyperbolic ts;
      VirtualTimeSource<Real_wp>* fsrc = this->GetNewTimeSource();
      ts.Init(fsrc, pb.GetFrequency(), this->epsilon_time, t0);
      std::vector<double> pulse3(nsteps);
      for (int n = 0; n < nsteps; n++) {
        double t = t0 + n * dt + dt;
        Real_wp p = 0;
        ts.EvaluateDerivative(t, 3, p);
        pulse3[n] = (t >= this->tlimit_source) ? 0.0 : p;
      }
      write_raw(outdir + "/pulse3.f64", pulse3.data(), pulse3.size());
    }

    // Operator product y = beta*y0 + alpha*Kh*x through the reference's
    // VirtualMatrix::MltAddVector (assemble = false, as ApplyOperatorKh does).
    if (!xfile.empty()) {
      std::vector<double> xv = read_f64(xfile);
      if ((int)xv.size() != ndof) { fprintf(stderr, "x has %zu entries, ndof %d\n", xv.size(), ndof); exit(2); }
      VectReal_wp x(ndof), y(ndof), ax(ndof);
      for (int i = 0; i < ndof; i++) x(i) = xv[i];
      if (!y0file.empty()) {
        std::vector<double> yv = read_f64(y0file);
        for (int i = 0; i < ndof; i++) y(i) = yv[i];
      } else {
        y.Fill(0.0);
      }
      this->Glob_mat_Kh->MltAddVector(Real_wp(alpha), x, Real_wp(beta), y, false);
      write_raw(outdir + "/kh_y.f64", y.GetData(), ndof);
      ax.Fill(0.0);
      this->Glob_mat_Kh->MltAddVector(Real_wp(1), x, Real_wp(0), ax, false);
      write_raw(outdir + "/kh_ax.f64", ax.GetData(), ndof);
    }

    FILE* f = fopen((outdir + "/meta.txt").c_str(), "w");
    fprintf(f, "n_elt %d\nn_dof %d\norder %d\nnq %d\n", ne, ndof, r, Q);
    fprintf(f, "dt %.17g\nt0 %.17g\ntf %.17g\nnsteps %d\n", dt, t0, tf, nsteps);
    fprintf(f, "tlimit_source %.17g\nepsilon_time %.17g\nfrequency %.17g\n",
            (double)this->tlimit_source, (double)this->epsilon_time, (double)pb.GetFrequency());
    fprintf(f, "n_src %d\n", (int)F.GetM());
    fclose(f);
  }

  void Record(int n, const Real_wp& t, Vector<Real_wp>& u) {
    if (record_norms) {
      norms.push_back(this->GetNormeSolution(u));
      times.push_back(t);
    }
    if (snaps.count(n)) {
      char name[64];
      snprintf(name, sizeof(name), "/u_%06d.f64", n);
      write_raw(outdir + name, u.GetData(), u.GetM());
    }
    last_n = n;
  }

  void GiveIterate(int n, const Real_wp& t, Vector<Real_wp>& u) override {
    if (!dumped) {
      DumpStatic();
      dumped = true;
      loop_start = std::chrono::steady_clock::now();
    }
    Record(n, t, u);
    VarInstationary_Base::GiveIterate(n, t, u);
  }

  void GiveFinalIterate(int n, const Real_wp& t, Vector<Real_wp>& u) override {
    loop_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - loop_start).count();
    Record(n, t, u);
    char name[64];
    snprintf(name, sizeof(name), "/u_final.f64");
    write_raw(outdir + name, u.GetData(), u.GetM());
    VarInstationary_Base::GiveFinalIterate(n, t, u);
  }
};

int main(int argc, char** argv) {
  InitMontjoie(argc, argv);
  if (argc < 3) {
    fprintf(stderr, "usage: ref_dump deck.ini outdir [options]\n");
    return 2;
  }
  std::string deck = argv[1];
  DumpingProblem* pb = new DumpingProblem();
  pb->outdir = argv[2];
  for (int i = 3; i < argc; i++) {
    std::string a = argv[i];
    auto next = [&]() { return std::string(argv[++i]); };
    if (a == "--x") pb->xfile = next();
    else if (a == "--y0") pb->y0file = next();
    else if (a == "--alpha") pb->alpha = atof(next().c_str());
    else if (a == "--beta") pb->beta = atof(next().c_str());
    else if (a == "--no-norms") pb->record_norms = false;
    else if (a == "--snaps") {
      std::stringstream ss(next());
      std::string tok;
      while (std::getline(ss, tok, ',')) pb->snaps.insert(atoi(tok.c_str()));
    }
  }
  std::string type_element, type_equation;
  getElement_Equation(deck, type_element, type_equation);
  auto t_start = std::chrono::steady_clock::now();
  pb->RunAll(deck, type_element, type_equation);
  double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();

  FILE* f = fopen((pb->outdir + "/run.txt").c_str(), "w");
  fprintf(f, "loop_seconds %.6f\ntotal_seconds %.6f\nlast_n %d\n", pb->loop_seconds, total, pb->last_n);
  fclose(f);
  if (pb->record_norms) {
    write_raw(pb->outdir + "/norms.f64", pb->norms.data(), pb->norms.size());
    write_raw(pb->outdir + "/times.f64", pb->times.data(), pb->times.size());
  }
  delete pb;
  return FinalizeMontjoie();
}
