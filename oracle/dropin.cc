// Test infrastructure only: the proof that the drop-in binding of
// INTEGRATION.md compiles against the reference's own headers and links with
// the product library (oracle/Makefile, target `dropin`; compiled where the
// reference sources lie, never copied).
//
// The two code blocks of INTEGRATION.md sections 1 and 2 appear here verbatim
// (tests/test_host_setup.py checks it):
//   1. GpuLaplaceMatrix, a FemMatrixFreeClass<double, LaplaceEquation<Dimension3> >
//      whose virtual product hook MltAddFree calls mj_op_mltadd;
//   2. the order-2 leap-frog of ApplySecondOrderScheme
//      (MONTJOIE/src/Instationary/VarInstationary.cxx:1479-1514) as one mj_lf_run.
// GpuAcousticProblem installs the first as Glob_mat_Kh through the virtual
// ComputeStiffnessMatrix (VarInstationary.cxx:1303-1313), so the reference's
// own RunAll drives the GPU operator; --gpu-loop also runs the second.
//
// Usage: dropin deck.ini [--gpu-loop [4]]     (needs a CUDA device to run)

#define MONTJOIE_WITH_TWO_DIM
#define MONTJOIE_WITH_THREE_DIM
#define MONTJOIE_WITH_NODAL_H1
#define MONTJOIE_WITH_NODAL_DG
#define SELDON_WITH_PRECONDITIONING
#define MONTJOIE_WITH_TIME_REVERSAL

#include "Hyperbolic/Acoustic/MontjoieAcoustic.hxx"
#include "Elliptic/Helmholtz/ProdMatVectHelmholtz.cxx"
#include "Computation/ProdMatVectScalarH1.cxx"

#include <cstdio>
#include <string>
#include <vector>

using namespace Montjoie;

// The Amos Bessel / Lambert-W Fortran routines are off the acoustic path and
// no Fortran compiler is available: link stubs that abort if ever reached.
extern "C" {
void cbesj_(const void*, const double*, int*, int*, void*, int*, int*) { abort(); }
void cbesy_(const void*, const double*, int*, int*, void*, int*, void*, int*) { abort(); }
void cbesk_(const void*, const double*, int*, int*, void*, int*, int*) { abort(); }
void lambert_(const double*, double*) { abort(); }
}

// ---- INTEGRATION.md, section 1 (verbatim) ----
#include "montjoie_gb300.h"

class GpuLaplaceMatrix : public FemMatrixFreeClass<double, LaplaceEquation<Dimension3> > {
  mj_op* op_ = nullptr;
 public:
  GpuLaplaceMatrix(const EllipticProblem<LaplaceEquation<Dimension3> >& var)
    : FemMatrixFreeClass<double, LaplaceEquation<Dimension3> >(var) {
    const int ne = var.mesh.GetNbElt(), r = var.GetReferenceElement(0).GetOrder();
    const int Q = (r + 1) * (r + 1) * (r + 1);
    std::vector<int32_t> nodle((size_t)ne * Q);
    std::vector<double> fac((size_t)ne * Q * 6);
    for (int e = 0; e < ne; e++) {
      IVect nod = var.GetDofNumberOnElement(e);                 // NumberMap connectivity
      const auto& Fb = var.GetReferenceElement(e);
      const int nb = var.Glob_matMass_Bh(e).GetM();             // 1 when affine + uniform media
      for (int j = 0; j < Q; j++) {
        nodle[(size_t)e * Q + j] = nod(j);
        const auto& m = var.Glob_matMass_Bh(e)(nb == 1 ? 0 : j); // VarHelmholtz.cxx:95-123
        const double w = (nb == 1) ? Fb.WeightsND(j) : 1.0;
        double* o = &fac[((size_t)e * Q + j) * 6];
        o[0] = w * m(0, 0); o[1] = w * m(0, 1); o[2] = w * m(0, 2);
        o[3] = w * m(1, 1); o[4] = w * m(1, 2); o[5] = w * m(2, 2);
      }
    }
    mj_mesh_desc mesh{r, ne, var.GetNbDof(), nodle.data()};
    mj_geom_desc geom{fac.data(), nullptr};
    if (mj_op_create(&mesh, &geom, MJ_FP64, &op_) != MJ_OK) { cout << mj_last_error() << endl; abort(); }
  }
  ~GpuLaplaceMatrix() { mj_op_destroy(op_); }
  mj_op* op() const { return op_; }                         // for the time loop of section 2

  // The virtual product hook FemMatrixFreeClass_Base<T>::MltAddFree (FemMatrixFreeClass.hxx:281-287,
  // Laplace's own in VarLaplace.hxx:383-399): Y += A X, Y zeroed by the caller
  // (FemMatrixFreeClass.cxx:1088-1101).  MltAddVector(alpha, X, beta, Y, assemble), which
  // ApplyOperatorKh calls, is not virtual; it reaches the product through this hook.
  using FemMatrixFreeClass<double, LaplaceEquation<Dimension3> >::MltAddFree;
  void MltAddFree(const GlobalGenericMatrix<double>& nat_mat, const SeldonTranspose& trans, int lvl,
                  const Vector<double>& X, Vector<double>& Y) const override {
    if (mj_op_mltadd(op_, 1.0, X.GetData(), 1.0, Y.GetData()) != MJ_OK) { cout << mj_last_error() << endl; abort(); }
  }
};
// ---- end of section 1 ----

class GpuAcousticProblem : public HyperbolicProblem<AcousticEquation<Dimension3> > {
 public:
  mj_op* gpu_kh_op = nullptr;  // the operator of Glob_mat_Kh, which the loop of section 2 runs on

  // Glob_mat_Kh on the GPU (VarInstationary_Base::ComputeStiffnessMatrix,
  // VarInstationary.cxx:1303-1313); its operator also runs the loop of section 2.
  void ComputeStiffnessMatrix() override {       // in a HyperbolicProblem<AcousticEquation<Dimension3> > subclass
    if (this->Glob_mat_Kh != NULL) delete this->Glob_mat_Kh;
    GpuLaplaceMatrix* kh = new GpuLaplaceMatrix(this->var_harmonic);
    gpu_kh_op = kh->op();
    this->Glob_mat_Kh = kh;
  }

  // The whole order-2 run on the GPU from U0, dU0_dt; U0 receives the final iterate.
  void RunLeapFrogOnGpu(VectReal_wp& U0, VectReal_wp& dU0_dt) {
    const int N = this->var_harmonic.GetNbDof();
    // ---- INTEGRATION.md, section 2 (verbatim) ----
    VectReal_wp D(N), invD(N), ones(N); ones.Fill(1.0); D.Fill(0.0); invD.Fill(1.0);
    ApplyOperatorDh(1.0, 0.0, ones, 0.0, D);        // lumped mass
    SolveOperatorDhPlusdtSh(invD);                   // 1/D as the scheme uses it
    const int nsteps = toInteger(ceil(abs(final_time - initial_time) / deltat));
    std::vector<double> pulse(nsteps);               // p(t_n + dt), zero from tlimit_source on
    for (int n = 0; n < nsteps; n++) {
      double t = initial_time + n * deltat + deltat, p = 0;
      if (t < tlimit_source) SourceOnlyTime(t, 1, p);
      pulse[n] = p;
    }
    std::vector<int32_t> src_idx(sparse_vector_source.GetM());
    for (int i = 0; i < sparse_vector_source.GetM(); i++) src_idx[i] = sparse_vector_source.Index(i);
    mj_lf_desc d{deltat, D.GetData(), invD.GetData(), (int)src_idx.size(), src_idx.data(),
                 sparse_vector_source.GetData(), nsteps, pulse.data(), nullptr, 0, 0, nullptr, nullptr};
    mj_lf* lf; mj_lf_create(gpu_kh_op, &d, &lf);
    mj_lf_run(lf, U0.GetData(), dU0_dt.GetData(), nsteps, U0.GetData(), nullptr, nullptr, 0);
    mj_lf_destroy(lf);
    // ---- end of section 2 ----
  }

  // The same run with the order-4 modified-equation leap-frog.
  void RunLeapFrog4OnGpu(VectReal_wp& U0, VectReal_wp& dU0_dt) {
    const int N = this->var_harmonic.GetNbDof();
    VectReal_wp D(N), invD(N), ones(N); ones.Fill(1.0); D.Fill(0.0); invD.Fill(1.0);
    ApplyOperatorDh(1.0, 0.0, ones, 0.0, D);
    SolveOperatorDhPlusdtSh(invD);
    const int nsteps = toInteger(ceil(abs(final_time - initial_time) / deltat));
    std::vector<double> pulse(nsteps);
    for (int n = 0; n < nsteps; n++) {
      double t = initial_time + n * deltat + deltat, p = 0;
      if (t < tlimit_source) SourceOnlyTime(t, 1, p);
      pulse[n] = p;
    }
    std::vector<int32_t> src_idx(sparse_vector_source.GetM());
    for (int i = 0; i < sparse_vector_source.GetM(); i++) src_idx[i] = sparse_vector_source.Index(i);
    mj_lf_desc d{deltat, D.GetData(), invD.GetData(), (int)src_idx.size(), src_idx.data(),
                 sparse_vector_source.GetData(), nsteps, pulse.data(), nullptr, 0, 0, nullptr, nullptr};
    mj_lf* lf; mj_lf_create(gpu_kh_op, &d, &lf);
    // ---- INTEGRATION.md, section 2, order 4 (verbatim) ----
    std::vector<double> pulse_d2(nsteps);
    for (int n = 0; n < nsteps; n++) {
      double t = initial_time + n * deltat + deltat, p = 0;
      if (t < tlimit_source) SourceOnlyTime(t, 3, p);
      pulse_d2[n] = p;
    }
    mj_lf_set_scheme(lf, 4, nsteps, pulse_d2.data());    // before mj_lf_init / mj_lf_run
    // ---- end of order 4 ----
    mj_lf_run(lf, U0.GetData(), dU0_dt.GetData(), nsteps, U0.GetData(), nullptr, nullptr, 0);
    mj_lf_destroy(lf);
  }
};

int main(int argc, char** argv) {
  InitMontjoie(argc, argv);
  if (argc < 2) {
    fprintf(stderr, "usage: dropin deck.ini [--gpu-loop [4]]\n");
    return 2;
  }
  std::string deck = argv[1], type_element, type_equation;
  getElement_Equation(deck, type_element, type_equation);
  GpuAcousticProblem* pb = new GpuAcousticProblem();
  pb->RunAll(deck, type_element, type_equation);  // the reference's loop, Kh on the GPU
  if (argc > 2 && std::string(argv[2]) == "--gpu-loop") {
    VectReal_wp U0(pb->var_harmonic.GetNbDof()), dU0(pb->var_harmonic.GetNbDof());
    U0.Fill(0.0);
    dU0.Fill(0.0);
    if (argc > 3 && std::string(argv[3]) == "4") pb->RunLeapFrog4OnGpu(U0, dU0);
    else pb->RunLeapFrogOnGpu(U0, dU0);
    printf("gpu loop: |u_final| = %.17g\n", Norm2(U0));
  }
  delete pb;
  return FinalizeMontjoie();
}
