// Test program for the C++ facade (include/pinocchio_gb300.hpp): builds a
// 3-joint chain, runs rneaInParallel / abaInParallel on host column-major
// matrices and prints the max |ABA(RNEA(a)) - a|; then the single calls
// rnea / aba / crba / computeRNEADerivatives / computeABADerivatives over a Data
// (ABA(RNEA(a)) = a, the ddq of the derivatives, Minv M = I, M of both algorithms).  A minimal column-major
// matrix type stands in for Eigen::MatrixXd (same rows/cols/data interface).
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "../../include/pinocchio_gb300.hpp"

struct Mat {
  long r, c;
  std::vector<double> d;
  Mat(long rows, long cols) : r(rows), c(cols), d(rows * cols, 0.0) {}
  long rows() const { return r; }
  long cols() const { return c; }
  const double* data() const { return d.data(); }
  double* data() { return d.data(); }
};

// Overload resolution of the external-force calls next to the plain ones (compiled,
// not run: these take device pointers).
[[maybe_unused]] static void fext_overloads_resolve(const pinocchio_gb300::Model& m, double* q, double* x, double* f,
                                                    double* o1, double* o2, double* o3) {
  const pinocchio_gb300::ExternalForces fe{f};
  pinocchio_gb300::rnea(m, GB_FP64, 1, q, x, x, o1);
  pinocchio_gb300::rnea(m, GB_FP64, 1, q, x, x, fe, o1);
  pinocchio_gb300::computeStaticTorque(m, GB_MIXED, 1, q, fe, o1);
  pinocchio_gb300::aba(m, GB_FP64, 1, q, x, x, o1, GB_WORLD);
  pinocchio_gb300::aba(m, GB_FP64, 1, q, x, x, fe, o1, GB_WORLD);
  pinocchio_gb300::computeRNEADerivatives(m, GB_FP64, 1, q, x, x, o1, o2, o3);
  pinocchio_gb300::computeRNEADerivatives(m, GB_FP64, 1, q, x, x, fe, o1, o2, o3);
  pinocchio_gb300::computeABADerivatives(m, GB_MIXED, 1, q, x, x, o1, o2, o3);
  pinocchio_gb300::computeABADerivatives(m, GB_MIXED, 1, q, x, x, fe, o1, o2, o3);
  pinocchio_gb300::forwardDynamics(m, GB_FP64, 1, q, x, x, 2, f, f, o1, o2);
  pinocchio_gb300::impulseDynamics(m, GB_FP64, 1, q, x, 2, f, o1, o2, 0.5);
  pinocchio_gb300::computeKKTContactDynamicMatrixInverse(m, 1, q, 2, f, o1, 1e-6);
}

int main() {
  pinocchio_gb300::ModelTables t;
  t.parents = {0, 0, 1, 2};
  t.jtype = {GB_JOINT_NONE, GB_JOINT_RZ, GB_JOINT_RY, GB_JOINT_RX};
  t.placement.assign(4 * 12, 0.0);
  t.inertia.assign(4 * 10, 0.0);
  for (int i = 0; i < 4; ++i) {
    double* P = &t.placement[12 * i];
    P[0] = P[4] = P[8] = 1.0;
    P[11] = i > 0 ? 0.25 : 0.0;
    double* Y = &t.inertia[10 * i];
    if (i > 0) { Y[0] = 1.0 + i; Y[3] = 0.1; Y[4] = 0.02; Y[6] = 0.03; Y[9] = 0.04; }
  }
  try {
    pinocchio_gb300::Model model(t);
    pinocchio_gb300::ModelPool pool(model, 4);
    const long B = 257;
    Mat q(model.nq, B), v(model.nv, B), a(model.nv, B), tau(model.nv, B), a2(model.nv, B);
    for (long k = 0; k < model.nq * B; ++k) q.d[k] = std::sin(0.37 * k);
    for (long k = 0; k < model.nv * B; ++k) { v.d[k] = std::cos(0.11 * k); a.d[k] = std::sin(0.23 * k + 1.0); }
    pinocchio_gb300::rneaInParallel(4, pool, q, v, a, tau);
    pinocchio_gb300::abaInParallel(4, pool, q, v, tau, a2);
    double err = 0.0;
    for (long k = 0; k < model.nv * B; ++k) err = std::fmax(err, std::fabs(a2.d[k] - a.d[k]));
    std::printf("roundtrip_max_abs_err %.3e\n", err);
    try {
      pinocchio_gb300::rneaInParallel(5, pool, q, v, a, tau);
      std::printf("expected an exception\n");
      return 2;
    } catch (const std::invalid_argument& e) {
      std::printf("pool_check_ok %s\n", e.what());
    }
    if (err >= 1e-10) return 1;

    // the reference's single-call signatures over a device-batched Data: host inputs,
    // a device input (data.tau of a previous call), outputs into caller matrices
    pinocchio_gb300::Data data(model), data2(model);
    const pinocchio_gb300::DeviceMatrix& tau_d = pinocchio_gb300::rnea(model, data, q, v, a);
    Mat tau2(model.nv, B), a3(model.nv, B);
    tau_d.copyToHost(tau2);
    double e1 = 0.0;
    for (long k = 0; k < model.nv * B; ++k) e1 = std::fmax(e1, std::fabs(tau2.d[k] - tau.d[k]));
    pinocchio_gb300::aba(model, data2, q, v, data.tau).copyToHost(a3);  // device input
    double e2 = 0.0;
    for (long k = 0; k < model.nv * B; ++k) e2 = std::fmax(e2, std::fabs(a3.d[k] - a.d[k]));
    const long nn = static_cast<long>(model.nv) * model.nv;
    Mat dq(nn, B), dv(nn, B), Minv(nn, B), Mup(nn, B), ddq(model.nv, B);
    pinocchio_gb300::computeABADerivatives(model, data, q, v, tau2, dq, dv, Minv);
    data.ddq.copyToHost(ddq);
    double e3 = 0.0;
    for (long k = 0; k < model.nv * B; ++k) e3 = std::fmax(e3, std::fabs(ddq.d[k] - a.d[k]));
    pinocchio_gb300::crba(model, data, q).copyToHost(Mup);
    double e4 = 0.0;  // Minv * M = I per configuration (M from its upper triangle)
    const int n = model.nv;
    for (long b = 0; b < B; ++b) {
      const double* Mi = &Minv.d[nn * b];
      const double* Mu = &Mup.d[nn * b];
      for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) {
          double s = 0.0;
          for (int k = 0; k < n; ++k) s += Mi[r * n + k] * (k <= c ? Mu[k * n + c] : Mu[c * n + k]);
          e4 = std::fmax(e4, std::fabs(s - (r == c ? 1.0 : 0.0)));
        }
    }
    pinocchio_gb300::computeRNEADerivatives(model, data, q, v, a);
    Mat M2(nn, B);
    data.M.copyToHost(M2);
    double e5 = 0.0;
    for (long k = 0; k < nn * B; ++k) e5 = std::fmax(e5, std::fabs(M2.d[k] - Mup.d[k]));
    pinocchio_gb300::checkNumeric(model);
    std::printf("single_calls rnea %.3e aba %.3e ddq %.3e minv_m %.3e M %.3e\n", e1, e2, e3, e4, e5);

    // constraintDynamics: no constraint gives ABA; a point contact at the chain's tip solved
    // undamped equals the proximal iterations with mu > 0 run to convergence
    std::vector<pinocchio_gb300::RigidConstraintModel> none;
    std::vector<pinocchio_gb300::RigidConstraintData> none_d;
    pinocchio_gb300::ProximalSettings ps0;
    Mat a4(model.nv, B), c1(model.nv, B), c2(model.nv, B);
    pinocchio_gb300::constraintDynamics(model, data, q, v, tau2, none, none_d, ps0).copyToHost(a4);
    double e6 = 0.0;
    for (long k = 0; k < model.nv * B; ++k) e6 = std::fmax(e6, std::fabs(a4.d[k] - a.d[k]));
    const double tip[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0.05, 0.0, 0.1};
    std::vector<pinocchio_gb300::RigidConstraintModel> cm{
        pinocchio_gb300::RigidConstraintModel(GB_CONTACT_3D, model, 3, tip, GB_FRAME_LOCAL)};
    std::vector<pinocchio_gb300::RigidConstraintData> cd{pinocchio_gb300::RigidConstraintData(cm[0])};
    pinocchio_gb300::constraintDynamics(model, data, q, v, tau2, cm, cd, ps0).copyToHost(c1);
    pinocchio_gb300::ProximalSettings ps1(1e-12, 1e-6, 200);
    pinocchio_gb300::constraintDynamics(model, data, q, v, tau2, cm, cd, ps1).copyToHost(c2);
    double e7 = 0.0, s7 = 0.0;
    for (long k = 0; k < model.nv * B; ++k) {
      e7 = std::fmax(e7, std::fabs(c1.d[k] - c2.d[k]));
      s7 = std::fmax(s7, std::fabs(c1.d[k]));
    }
    std::printf("constraint_dynamics aba %.3e prox %.3e iter %d lambda_rows %ld\n", e6, e7 / s7, ps1.iter,
                data.lambda_c.rows());
    if (!(e6 < 1e-10 && e7 < 1e-6 * s7 && ps1.iter > 1 && data.lambda_c.rows() == 3 && cd[0].size == 3)) return 6;
    // ContactCholeskyDecomposition at the configurations of crba: inverse() * matrix() = I and
    // getInverseMassMatrix() * M = I
    pinocchio_gb300::crba(model, data, q);
    pinocchio_gb300::ContactCholeskyDecomposition chol(model, cm);
    chol.compute(model, data, cm, cd, 1e-3);
    const int nk = chol.size();
    Mat K(static_cast<long>(nk) * nk, B), Ki(static_cast<long>(nk) * nk, B);
    chol.matrix().copyToHost(K);
    chol.inverse().copyToHost(Ki);
    double e8 = 0.0;
    for (long b = 0; b < B; ++b)
      for (int r = 0; r < nk; ++r)
        for (int c = 0; c < nk; ++c) {
          double t = 0.0;
          for (int k = 0; k < nk; ++k) t += Ki.d[b * nk * nk + r * nk + k] * K.d[b * nk * nk + k * nk + c];
          e8 = std::fmax(e8, std::fabs(t - (r == c ? 1.0 : 0.0)));
        }
    std::printf("contact_cholesky size %d dim %d kkt_inverse %.3e\n", nk, chol.constraintDim(), e8);
    if (!(nk == model.nv + 3 && chol.constraintDim() == 3 && e8 < 1e-8)) return 7;
    try {
      Mat bad(model.nq + 1, B);
      pinocchio_gb300::rnea(model, data, bad, v, a);
      std::printf("expected an exception\n");
      return 4;
    } catch (const std::invalid_argument& e) {
      std::printf("size_check_ok %s\n", e.what());
    }
    return (e1 < 1e-12 && e2 < 1e-10 && e3 < 1e-10 && e4 < 1e-10 && e5 < 1e-12) ? 0 : 5;
  } catch (const std::exception& e) {
    std::printf("error %s\n", e.what());
    return 3;
  }
}
