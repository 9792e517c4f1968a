// C++ facade over the C ABI with the argument shapes of the reference's batched
// dynamics entry points:
//   rneaInParallel(num_threads, pool, q, v, a, tau)   (algorithm/parallel/rnea.hpp:39-84)
//   abaInParallel(num_threads, pool, q, v, tau, a)    (algorithm/parallel/aba.hpp:40-84)
// the reference's single calls with their signatures, over a device-batched Data
// (one column of q, v, a, tau per configuration; a vector is a batch of one):
//   rnea(model, data, q, v, a)                    -> data.tau   (algorithm/rnea.hpp:37-42)
//   aba(model, data, q, v, tau, convention)       -> data.ddq   (algorithm/aba.hpp:41-47)
//   crba(model, data, q, convention)              -> data.M     (algorithm/crba.hpp:47-51)
//   computeRNEADerivatives(model, data, q, v, a)  -> data.dtau_dq, dtau_dv, M
//                                                    (algorithm/rnea-derivatives.hpp:120-260)
//   computeABADerivatives(model, data, q, v, tau) -> data.ddq_dq, ddq_dv, Minv, ddq
//                                                    (algorithm/aba-derivatives.hpp:52-310)
// and, for device-resident batches, the same functions over raw (batch, n) device arrays.
//
// Matrix arguments are any type with rows(), cols() and data() over contiguous
// column-major double storage -- Eigen::MatrixXd satisfies this, so a caller of
// the reference passes the same objects.  Errors are thrown as
// std::invalid_argument (size / pool errors, as PINOCCHIO_CHECK_ARGUMENT_SIZE
// does, include/pinocchio/macros.hpp:162-223) or std::runtime_error (device errors).
#ifndef PINOCCHIO_GB300_HPP
#define PINOCCHIO_GB300_HPP

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "pinocchio_gb300.h"

namespace pinocchio_gb300 {

inline void check(int rc) {
  if (rc == GB_OK) return;
  const std::string msg = gb_last_error();
  if (rc == GB_ERR_SIZE || rc == GB_ERR_POOL || rc == GB_ERR_INVALID_ARGUMENT || rc == GB_ERR_GRAVITY ||
      rc == GB_ERR_UNSUPPORTED)
    throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}

// A flattened kinematic tree (the ModelTpl tables the batched path reads).
struct ModelTables {
  std::vector<int> parents, jtype;  // joint 0 = universe (GB_JOINT_NONE)
  std::vector<double> placement;    // njoints x 12
  std::vector<double> inertia;      // njoints x 10
  std::vector<double> armature;     // nv
  double gravity[6] = {0, 0, -9.81, 0, 0, 0};
  std::vector<double> axis;         // njoints x 3: axes of the unaligned joints (empty: none)
  // mimic joints (gb_model_desc.mimic): per joint the joint it mimics (0: none), its scaling and
  // offset; empty: none
  std::vector<int> mimic;
  std::vector<double> mimic_scaling, mimic_offset;
};

class Model {
 public:
  explicit Model(const ModelTables& t) {
    gb_model_desc d{};
    d.njoints = static_cast<int>(t.parents.size());
    d.parents = t.parents.data();
    d.jtype = t.jtype.data();
    d.placement = t.placement.data();
    d.inertia = t.inertia.data();
    d.armature = t.armature.empty() ? nullptr : t.armature.data();
    d.nv_armature = static_cast<int>(t.armature.size());
    d.gravity = t.gravity;
    d.axis = t.axis.empty() ? nullptr : t.axis.data();
    d.mimic = t.mimic.empty() ? nullptr : t.mimic.data();
    d.mimic_scaling = t.mimic_scaling.empty() ? nullptr : t.mimic_scaling.data();
    d.mimic_offset = t.mimic_offset.empty() ? nullptr : t.mimic_offset.data();
    gb_model* m = nullptr;
    check(gb_model_create(&d, &m));
    handle_.reset(m, [](gb_model* p) { gb_model_destroy(p); });
    check(gb_model_dims(m, &nq, &nv, &njoints));
    check(gb_model_nv_extended(m, &nvExtended));
  }
  gb_model* get() const { return handle_.get(); }
  int nq = 0, nv = 0, njoints = 0, nvExtended = 0;

 private:
  std::shared_ptr<gb_model> handle_;
};

// ModelPool(model, size) (multibody/pool/model.hpp:19-165).
class ModelPool {
 public:
  ModelPool(const Model& model, long size) : model_(model) {
    gb_pool* p = nullptr;
    check(gb_pool_create(model.get(), size, &p));
    handle_.reset(p, [](gb_pool* q) { gb_pool_destroy(q); });
  }
  long size() const {
    long s = 0;
    check(gb_pool_size(handle_.get(), &s));
    return s;
  }
  void setPrecision(int precision) { check(gb_pool_set_precision(handle_.get(), precision)); }
  const Model& getModel() const { return model_; }
  gb_pool* get() const { return handle_.get(); }

 private:
  Model model_;
  std::shared_ptr<gb_pool> handle_;
};

namespace detail {
template <class M> void check_rows(const M& x, long rows, const char* name) {
  if (static_cast<long>(x.rows()) != rows)
    throw std::invalid_argument(std::string("wrong number of rows for ") + name);
}
}  // namespace detail

// q: nq x batch, v, a: nv x batch, tau: nv x batch (written), column-major host storage.
template <class MQ, class MV, class MA, class MT>
void rneaInParallel(std::size_t num_threads, ModelPool& pool, const MQ& q, const MV& v, const MA& a, MT& tau) {
  const Model& m = pool.getModel();
  detail::check_rows(q, m.nq, "q");
  detail::check_rows(v, m.nv, "v");
  detail::check_rows(a, m.nv, "a");
  detail::check_rows(tau, m.nv, "tau");
  if (q.cols() != v.cols() || q.cols() != a.cols() || q.cols() != tau.cols())
    throw std::invalid_argument("all batch matrices must have the same number of columns");
  check(gb_rnea_in_parallel(static_cast<long>(num_threads), pool.get(), static_cast<long>(q.cols()), q.data(),
                            v.data(), a.data(), tau.data()));
}

// q: nq x batch, v, tau: nv x batch, a: nv x batch (written); WORLD convention as the reference.
template <class MQ, class MV, class MT, class MA>
void abaInParallel(std::size_t num_threads, ModelPool& pool, const MQ& q, const MV& v, const MT& tau, MA& a) {
  const Model& m = pool.getModel();
  detail::check_rows(q, m.nq, "q");
  detail::check_rows(v, m.nv, "v");
  detail::check_rows(tau, m.nv, "tau");
  detail::check_rows(a, m.nv, "a");
  if (q.cols() != v.cols() || q.cols() != tau.cols() || q.cols() != a.cols())
    throw std::invalid_argument("all batch matrices must have the same number of columns");
  check(gb_aba_in_parallel(static_cast<long>(num_threads), pool.get(), static_cast<long>(q.cols()), q.data(),
                           v.data(), tau.data(), a.data()));
}

// ---- device-resident batches (pointers to device memory, GB_LAYOUT_INSTANCE) -------------------
inline void rnea(const Model& m, int precision, long batch, const double* q, const double* v, const double* a,
                 double* tau, void* stream = nullptr) {
  check(gb_rnea(m.get(), precision, GB_LAYOUT_INSTANCE, batch, q, v, a, tau, stream));
}
inline void aba(const Model& m, int precision, long batch, const double* q, const double* v, const double* tau,
                double* ddq, int convention = GB_LOCAL, void* stream = nullptr) {
  check(gb_aba(m.get(), precision, convention, GB_LAYOUT_INSTANCE, batch, q, v, tau, ddq, stream));
}
inline void crba(const Model& m, int precision, long batch, const double* q, double* M, int convention = GB_LOCAL,
                 void* stream = nullptr) {
  check(gb_crba(m.get(), precision, convention, GB_MATRIX_UPPER, GB_LAYOUT_INSTANCE, batch, q, M, nullptr, nullptr,
                stream));
}
inline void computeRNEADerivatives(const Model& m, int precision, long batch, const double* q, const double* v,
                                   const double* a, double* dtau_dq, double* dtau_dv, double* M,
                                   void* stream = nullptr) {
  check(gb_rnea_derivatives(m.get(), precision, GB_MATRIX_UPPER, GB_LAYOUT_INSTANCE, batch, q, v, a, dtau_dq, dtau_dv,
                            M, nullptr, stream));
}
inline void computeABADerivatives(const Model& m, int precision, long batch, const double* q, const double* v,
                                  const double* tau, double* ddq_dq, double* ddq_dv, double* Minv,
                                  void* stream = nullptr) {
  check(gb_aba_derivatives(m.get(), precision, GB_LAYOUT_INSTANCE, batch, q, v, tau, ddq_dq, ddq_dv, Minv, nullptr,
                           stream));
}

// ---- external forces: the reference's fext overloads (rnea.hxx:164-218, 448-489;
// aba.hxx:958-973; rnea-derivatives.hxx:550-633; aba-derivatives.hxx:463-541).
// `data` holds batch x njoints x 6 doubles on the device: per configuration, the
// force [linear; angular] on each joint in that joint's frame (joint 0 not read).
// A distinct type keeps these overloads apart from the ones without forces.
struct ExternalForces {
  const double* data;
};
inline void rnea(const Model& m, int precision, long batch, const double* q, const double* v, const double* a,
                 ExternalForces fext, double* tau, void* stream = nullptr) {
  check(gb_rnea_fext(m.get(), precision, GB_LAYOUT_INSTANCE, batch, q, v, a, fext.data, tau, stream));
}
inline void computeStaticTorque(const Model& m, int precision, long batch, const double* q, ExternalForces fext,
                                double* tau, void* stream = nullptr) {
  check(gb_static_torque(m.get(), precision, GB_LAYOUT_INSTANCE, batch, q, fext.data, tau, stream));
}
inline void aba(const Model& m, int precision, long batch, const double* q, const double* v, const double* tau,
                ExternalForces fext, double* ddq, int convention = GB_LOCAL, void* stream = nullptr) {
  check(gb_aba_fext(m.get(), precision, convention, GB_LAYOUT_INSTANCE, batch, q, v, tau, fext.data, ddq, stream));
}
inline void computeRNEADerivatives(const Model& m, int precision, long batch, const double* q, const double* v,
                                   const double* a, ExternalForces fext, double* dtau_dq, double* dtau_dv, double* M,
                                   void* stream = nullptr) {
  check(gb_rnea_derivatives_fext(m.get(), precision, GB_MATRIX_UPPER, GB_LAYOUT_INSTANCE, batch, q, v, a, fext.data,
                                 dtau_dq, dtau_dv, M, nullptr, stream));
}
inline void computeABADerivatives(const Model& m, int precision, long batch, const double* q, const double* v,
                                  const double* tau, ExternalForces fext, double* ddq_dq, double* ddq_dv, double* Minv,
                                  void* stream = nullptr) {
  check(gb_aba_derivatives_fext(m.get(), precision, GB_LAYOUT_INSTANCE, batch, q, v, tau, fext.data, ddq_dq, ddq_dv,
                                Minv, nullptr, stream));
}

// ---- contact dynamics with a constraint Jacobian J (nc x nv row-major per configuration, device
// memory): forwardDynamics (contact-dynamics.hxx:81-165) and impulseDynamics (255-327)
inline void forwardDynamics(const Model& m, int precision, long batch, const double* q, const double* v,
                            const double* tau, int nc, const double* J, const double* gamma, double* ddq,
                            double* lambda_c, double inv_damping = 0.0, void* stream = nullptr) {
  check(gb_forward_dynamics(m.get(), precision, GB_LAYOUT_INSTANCE, batch, nc, q, v, tau, J, gamma, inv_damping, ddq,
                            lambda_c, stream));
}
inline void computeKKTContactDynamicMatrixInverse(const Model& m, long batch, const double* q, int nc, const double* J,
                                                  double* KKTMatrix_inv, double inv_damping = 0.0,
                                                  void* stream = nullptr) {
  check(gb_kkt_contact_inverse(m.get(), GB_FP64, GB_LAYOUT_INSTANCE, batch, nc, q, J, inv_damping, KKTMatrix_inv, stream));
}
inline void impulseDynamics(const Model& m, int precision, long batch, const double* q, const double* v_before, int nc,
                            const double* J, double* dq_after, double* impulse_c, double r_coeff = 0.0,
                            double inv_damping = 0.0, void* stream = nullptr) {
  check(gb_impulse_dynamics(m.get(), precision, GB_LAYOUT_INSTANCE, batch, nc, q, v_before, J, r_coeff, inv_damping,
                            dq_after, impulse_c, stream));
}
inline void computeMinverse(const Model& m, int precision, long batch, const double* q, double* Minv,
                            void* stream = nullptr) {
  check(gb_compute_minverse(m.get(), precision, GB_MATRIX_UPPER, GB_LAYOUT_INSTANCE, batch, q, Minv, stream));
}
inline void nonLinearEffects(const Model& m, int precision, long batch, const double* q, const double* v, double* nle,
                             void* stream = nullptr) {
  check(gb_nonlinear_effects(m.get(), precision, GB_LAYOUT_INSTANCE, batch, q, v, nle, stream));
}
inline void computeGeneralizedGravity(const Model& m, int precision, long batch, const double* q, double* g,
                                      void* stream = nullptr) {
  check(gb_generalized_gravity(m.get(), precision, GB_LAYOUT_INSTANCE, batch, q, g, stream));
}
// v, a, v_out, a_out may be null (placements only, or placements and velocities)
inline void forwardKinematics(const Model& m, int precision, long batch, const double* q, const double* v,
                              const double* a, double* oMi, double* v_out, double* a_out, void* stream = nullptr) {
  check(gb_forward_kinematics(m.get(), precision, GB_LAYOUT_INSTANCE, batch, q, v, a, oMi, v_out, a_out, stream));
}
inline void computeJointJacobians(const Model& m, int precision, long batch, const double* q, double* J,
                                  void* stream = nullptr) {
  check(gb_compute_joint_jacobians(m.get(), precision, GB_LAYOUT_INSTANCE, batch, q, J, stream));
}

// ---- the reference's single-call signatures over a device-batched Data -------------------------
inline void check_cuda(cudaError_t e, const char* where) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(where) + ": " + cudaGetErrorString(e));
}

// A column-major rows x cols matrix of doubles in device memory (owned).  Batched
// outputs hold one configuration per column: a vector output is n x batch, a matrix
// output (nv x nv per configuration, row-major as the reference's RowMatrixXs) is
// (nv * nv) x batch.
class DeviceMatrix {
 public:
  DeviceMatrix() = default;
  DeviceMatrix(const DeviceMatrix&) = delete;
  DeviceMatrix& operator=(const DeviceMatrix&) = delete;
  ~DeviceMatrix() {
    if (p_) cudaFree(p_);
  }
  long rows() const { return r_; }
  long cols() const { return c_; }
  double* data() { return p_; }
  const double* data() const { return p_; }
  // sets the size, reallocating only when it grows
  void resize(long rows, long cols) {
    const size_t n = static_cast<size_t>(rows) * static_cast<size_t>(cols);
    if (n > cap_) {
      if (p_) cudaFree(p_);
      p_ = nullptr;
      cap_ = 0;
      check_cuda(cudaMalloc(&p_, sizeof(double) * (n > 0 ? n : 1)), "DeviceMatrix");
      cap_ = n;
    }
    r_ = rows;
    c_ = cols;
  }
  // copies into any host matrix with the same rows / cols and contiguous column-major data()
  template <class M> void copyToHost(M& out, void* stream = nullptr) const {
    if (static_cast<long>(out.rows()) != r_ || static_cast<long>(out.cols()) != c_)
      throw std::invalid_argument("copyToHost: the destination has the wrong size");
    check_cuda(cudaMemcpyAsync(out.data(), p_, sizeof(double) * r_ * c_, cudaMemcpyDeviceToHost,
                               static_cast<cudaStream_t>(stream)),
               "copyToHost");
    check_cuda(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "copyToHost");
  }

 private:
  double* p_ = nullptr;
  long r_ = 0, c_ = 0;
  size_t cap_ = 0;
};

class ConstraintSet;

// The device-batched counterpart of DataTpl (multibody/data.hpp): the precision and
// stream of the calls and the outputs the reference keeps in data, for a batch of
// configurations.  The batch size is the number of columns of q in each call.
class Data {
 public:
  explicit Data(const Model& model, int precision = GB_FP64, void* stream = nullptr)
      : nq(model.nq), nv(model.nv), precision(precision), stream(stream) {}
  int nq, nv;
  int precision;
  void* stream;
  DeviceMatrix tau, ddq, M, dtau_dq, dtau_dv, ddq_dq, ddq_dv, Minv;
  DeviceMatrix lambda_c, prox_residuals;  // constraintDynamics: multipliers, (absolute, relative) residuals
  DeviceMatrix q_crba;                    // the configurations of the last crba (ContactCholeskyDecomposition::compute)
  std::shared_ptr<ConstraintSet> constraints;  // the models of initConstraintDynamics

  // a device pointer to the n x batch input x: x itself when it lives in device (or
  // managed) memory, else a copy in the input slot
  template <class X> const double* input(int slot, const X& x, long n, long batch, const char* name) {
    if (static_cast<long>(x.rows()) != n)
      throw std::invalid_argument(std::string("wrong number of rows for ") + name);
    if (static_cast<long>(x.cols()) != batch)
      throw std::invalid_argument(std::string("wrong number of columns for ") + name);
    const double* p = x.data();
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) == cudaSuccess &&
        (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged))
      return p;
    (void)cudaGetLastError();  // an unregistered host pointer may leave an error behind
    staged_[slot].resize(n, batch);
    check_cuda(cudaMemcpyAsync(staged_[slot].data(), p, sizeof(double) * n * batch, cudaMemcpyHostToDevice,
                               static_cast<cudaStream_t>(stream)),
               "input copy");
    return staged_[slot].data();
  }

 private:
  DeviceMatrix staged_[3];
};

// tau = RNEA(q, v, a) of every column (algorithm/rnea.hpp:37-42): data.tau (nv x batch)
template <class MQ, class MV, class MA>
const DeviceMatrix& rnea(const Model& m, Data& data, const MQ& q, const MV& v, const MA& a) {
  const long B = static_cast<long>(q.cols());
  const double* Q = data.input(0, q, m.nq, B, "q");
  const double* V = data.input(1, v, m.nv, B, "v");
  const double* A = data.input(2, a, m.nv, B, "a");
  data.tau.resize(m.nv, B);
  check(gb_rnea(m.get(), data.precision, GB_LAYOUT_INSTANCE, B, Q, V, A, data.tau.data(), data.stream));
  return data.tau;
}

// ddq = ABA(q, v, tau) of every column (algorithm/aba.hpp:41-47): data.ddq (nv x batch)
template <class MQ, class MV, class MT>
const DeviceMatrix& aba(const Model& m, Data& data, const MQ& q, const MV& v, const MT& tau,
                        int convention = GB_LOCAL) {
  const long B = static_cast<long>(q.cols());
  const double* Q = data.input(0, q, m.nq, B, "q");
  const double* V = data.input(1, v, m.nv, B, "v");
  const double* T = data.input(2, tau, m.nv, B, "tau");
  data.ddq.resize(m.nv, B);
  check(gb_aba(m.get(), data.precision, convention, GB_LAYOUT_INSTANCE, B, Q, V, T, data.ddq.data(), data.stream));
  return data.ddq;
}

// M(q) of every column, upper triangle (algorithm/crba.hpp:47-51): data.M ((nv * nv) x batch)
template <class MQ>
const DeviceMatrix& crba(const Model& m, Data& data, const MQ& q, int convention = GB_LOCAL) {
  const long B = static_cast<long>(q.cols());
  const double* Q = data.input(0, q, m.nq, B, "q");
  data.M.resize(static_cast<long>(m.nv) * m.nv, B);
  check(gb_crba(m.get(), data.precision, convention, GB_MATRIX_UPPER, GB_LAYOUT_INSTANCE, B, Q, data.M.data(), nullptr,
                nullptr, data.stream));
  data.q_crba.resize(m.nq, B);
  check_cuda(cudaMemcpyAsync(data.q_crba.data(), Q, sizeof(double) * m.nq * B, cudaMemcpyDeviceToDevice,
                             static_cast<cudaStream_t>(data.stream)),
             "crba");
  return data.M;
}

// dtau/dq, dtau/dv and M (upper) of every column (algorithm/rnea-derivatives.hpp:120-260):
// data.dtau_dq, data.dtau_dv, data.M ((nv * nv) x batch each) and data.tau
template <class MQ, class MV, class MA>
void computeRNEADerivatives(const Model& m, Data& data, const MQ& q, const MV& v, const MA& a) {
  const long B = static_cast<long>(q.cols());
  const double* Q = data.input(0, q, m.nq, B, "q");
  const double* V = data.input(1, v, m.nv, B, "v");
  const double* A = data.input(2, a, m.nv, B, "a");
  const long nn = static_cast<long>(m.nv) * m.nv;
  data.dtau_dq.resize(nn, B);
  data.dtau_dv.resize(nn, B);
  data.M.resize(nn, B);
  data.tau.resize(m.nv, B);
  check(gb_rnea_derivatives(m.get(), data.precision, GB_MATRIX_UPPER, GB_LAYOUT_INSTANCE, B, Q, V, A,
                            data.dtau_dq.data(), data.dtau_dv.data(), data.M.data(), data.tau.data(), data.stream));
}

// ddq/dq, ddq/dv and Minv of every column (algorithm/aba-derivatives.hpp:52-310):
// data.ddq_dq, data.ddq_dv, data.Minv ((nv * nv) x batch each, Minv symmetric) and data.ddq
template <class MQ, class MV, class MT>
void computeABADerivatives(const Model& m, Data& data, const MQ& q, const MV& v, const MT& tau) {
  const long B = static_cast<long>(q.cols());
  const double* Q = data.input(0, q, m.nq, B, "q");
  const double* V = data.input(1, v, m.nv, B, "v");
  const double* T = data.input(2, tau, m.nv, B, "tau");
  const long nn = static_cast<long>(m.nv) * m.nv;
  data.ddq_dq.resize(nn, B);
  data.ddq_dv.resize(nn, B);
  data.Minv.resize(nn, B);
  data.ddq.resize(m.nv, B);
  check(gb_aba_derivatives(m.get(), data.precision, GB_LAYOUT_INSTANCE, B, Q, V, T, data.ddq_dq.data(),
                           data.ddq_dv.data(), data.Minv.data(), data.ddq.data(), data.stream));
}

// The overloads writing into caller matrices (aba-derivatives.hpp:99-130): each output is
// (nv * nv) x batch (one row-major nv x nv matrix per column), in device or host memory.
template <class MQ, class MV, class MT, class M1, class M2, class M3>
void computeABADerivatives(const Model& m, Data& data, const MQ& q, const MV& v, const MT& tau, M1& ddq_dq,
                           M2& ddq_dv, M3& dtau) {
  computeABADerivatives(m, data, q, v, tau);
  const long nn = static_cast<long>(m.nv) * m.nv;
  auto out = [&](const DeviceMatrix& src, auto& dst, const char* name) {
    if (static_cast<long>(dst.rows()) != nn || static_cast<long>(dst.cols()) != src.cols())
      throw std::invalid_argument(std::string("wrong size for ") + name);
    check_cuda(cudaMemcpyAsync(dst.data(), src.data(), sizeof(double) * nn * src.cols(), cudaMemcpyDefault,
                               static_cast<cudaStream_t>(data.stream)),
               name);
  };
  out(data.ddq_dq, ddq_dq, "ddq_dq");
  out(data.ddq_dv, ddq_dv, "ddq_dv");
  out(data.Minv, dtau, "Minv");
  check_cuda(cudaStreamSynchronize(static_cast<cudaStream_t>(data.stream)), "computeABADerivatives");
}

// ---- constraintDynamics (algorithm/constrained-dynamics.hpp:90-110) ---------------------------
// RigidConstraintModel(type, model, joint1_id, joint1_placement, joint2_id, joint2_placement,
// reference_frame) (algorithm/contact-info.hpp:236-262) in the flattened gb_constraint_desc form:
// placements are 12 doubles (R row-major, then t); Kp, Kd and the desired acceleration are public.
struct RigidConstraintModel : gb_constraint_desc {
  RigidConstraintModel(int contact_type, const Model& m, int joint1, const double* joint1_placement, int joint2,
                       const double* joint2_placement, int frame = GB_FRAME_LOCAL)
      : gb_constraint_desc{} {
    (void)m;
    type = contact_type;
    reference_frame = frame;
    joint1_id = joint1;
    joint2_id = joint2;
    for (int k = 0; k < 12; ++k) {
      this->joint1_placement[k] = joint1_placement ? joint1_placement[k] : (k == 0 || k == 4 || k == 8 ? 1.0 : 0.0);
      this->joint2_placement[k] = joint2_placement ? joint2_placement[k] : (k == 0 || k == 4 || k == 8 ? 1.0 : 0.0);
    }
  }
  RigidConstraintModel(int contact_type, const Model& m, int joint1, const double* joint1_placement,
                       int frame = GB_FRAME_LOCAL)
      : RigidConstraintModel(contact_type, m, joint1, joint1_placement, 0, nullptr, frame) {}
  int size() const { return type == GB_CONTACT_3D ? 3 : 6; }
};
// RigidConstraintData: after a call, this constraint's rows of data.lambda_c (its force in its frame)
struct RigidConstraintData {
  explicit RigidConstraintData(const RigidConstraintModel& c) : size(c.size()) {}
  int row = 0, size = 0;
};
// ProximalSettings (algorithm/proximal.hpp:22-110); after a call, iter and the residuals are the
// largest over the batch
struct ProximalSettings {
  ProximalSettings() = default;
  ProximalSettings(double accuracy, double mu_, int max_iter_)
      : absolute_accuracy(accuracy), relative_accuracy(accuracy), mu(mu_), max_iter(max_iter_) {}
  ProximalSettings(double absolute, double relative, double mu_, int max_iter_)
      : absolute_accuracy(absolute), relative_accuracy(relative), mu(mu_), max_iter(max_iter_) {}
  double absolute_accuracy = 1e-12, relative_accuracy = 1e-12, mu = 0.0;
  int max_iter = 1;
  int iter = 0;
  double absolute_residual = -1.0, relative_residual = -1.0;
};

// The constraint models of initConstraintDynamics on the device (gb_constraint_set), kept in Data
class ConstraintSet {
 public:
  ConstraintSet(const Model& m, const std::vector<RigidConstraintModel>& cms) : descs_(cms.begin(), cms.end()) {
    check(gb_constraint_set_create(m.get(), static_cast<int>(descs_.size()), descs_.data(), &h_));
    check(gb_constraint_set_dims(h_, nullptr, &dim_));
  }
  ConstraintSet(const ConstraintSet&) = delete;
  ConstraintSet& operator=(const ConstraintSet&) = delete;
  ~ConstraintSet() { gb_constraint_set_destroy(h_); }
  bool same(const std::vector<RigidConstraintModel>& cms) const {
    if (cms.size() != descs_.size()) return false;
    for (size_t k = 0; k < cms.size(); ++k)
      if (std::memcmp(static_cast<const gb_constraint_desc*>(&cms[k]), &descs_[k], sizeof(gb_constraint_desc)) != 0)
        return false;
    return true;
  }
  const gb_constraint_set* get() const { return h_; }
  int dim() const { return dim_; }

 private:
  std::vector<gb_constraint_desc> descs_;
  gb_constraint_set* h_ = nullptr;
  int dim_ = 0;
};

// initConstraintDynamics(model, data, contact_models) (constrained-dynamics.hxx:21-60)
inline void initConstraintDynamics(const Model& m, Data& data, const std::vector<RigidConstraintModel>& cms) {
  data.constraints.reset(new ConstraintSet(m, cms));
}

// ddq = constraintDynamics(model, data, q, v, tau, contact_models, contact_datas, settings) of every
// column: data.ddq (nv x batch), data.lambda_c (constraint_dim x batch); contact_datas[k] gets its
// rows; settings.iter and the residuals the largest over the batch (this reads them back: the call
// synchronises data.stream).
template <class MQ, class MV, class MT>
const DeviceMatrix& constraintDynamics(const Model& m, Data& data, const MQ& q, const MV& v, const MT& tau,
                                       const std::vector<RigidConstraintModel>& contact_models,
                                       std::vector<RigidConstraintData>& contact_datas, ProximalSettings& settings) {
  if (contact_models.size() != contact_datas.size())
    throw std::invalid_argument("The contact models and data do not have the same vector size.");
  if (!data.constraints || !data.constraints->same(contact_models)) initConstraintDynamics(m, data, contact_models);
  const long B = static_cast<long>(q.cols());
  const double* Q = data.input(0, q, m.nq, B, "q");
  const double* V = data.input(1, v, m.nv, B, "v");
  const double* T = data.input(2, tau, m.nv, B, "tau");
  const int nc = data.constraints->dim();
  data.ddq.resize(m.nv, B);
  data.lambda_c.resize(nc, B);
  data.prox_residuals.resize(2, B);
  std::vector<int> iters(static_cast<size_t>(B > 0 ? B : 1));
  int* d_iters = nullptr;
  check_cuda(cudaMalloc(&d_iters, sizeof(int) * iters.size()), "constraintDynamics");
  const gb_proximal_settings ps{settings.absolute_accuracy, settings.relative_accuracy, settings.mu, settings.max_iter};
  const int rc = gb_constraint_dynamics(m.get(), data.precision, data.constraints->get(), &ps, GB_LAYOUT_INSTANCE, B,
                                        Q, V, T, data.ddq.data(), nc > 0 ? data.lambda_c.data() : nullptr, d_iters,
                                        data.prox_residuals.data(), data.stream);
  std::vector<double> res(static_cast<size_t>(2 * (B > 0 ? B : 1)));
  cudaError_t e = cudaSuccess;
  if (rc == GB_OK && B > 0) {
    e = cudaMemcpyAsync(iters.data(), d_iters, sizeof(int) * B, cudaMemcpyDeviceToHost,
                        static_cast<cudaStream_t>(data.stream));
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(res.data(), data.prox_residuals.data(), sizeof(double) * 2 * B, cudaMemcpyDeviceToHost,
                          static_cast<cudaStream_t>(data.stream));
    if (e == cudaSuccess) e = cudaStreamSynchronize(static_cast<cudaStream_t>(data.stream));
  }
  cudaFree(d_iters);
  check(rc);
  check_cuda(e, "constraintDynamics");
  settings.iter = 0;
  settings.absolute_residual = settings.relative_residual = 0.0;
  for (long b = 0; b < B; ++b) {
    settings.iter = std::max(settings.iter, iters[b]);
    settings.absolute_residual = std::max(settings.absolute_residual, res[2 * b]);
    settings.relative_residual = std::max(settings.relative_residual, res[2 * b + 1]);
  }
  int row = 0;
  for (size_t k = 0; k < contact_datas.size(); ++k) {
    contact_datas[k].row = row;
    contact_datas[k].size = contact_models[k].size();
    row += contact_models[k].size();
  }
  return data.ddq;
}

// ContactCholeskyDecomposition(model, contact_models) (algorithm/contact-cholesky.hpp:107-470) over
// a batch: compute(model, data, contact_models, contact_datas, mu) factorises the KKT matrix
// [[-mu I, J], [J^T, M]] at the configurations of the last crba(model, data, q) (whose data.M the
// reference's compute reads); the accessors are device matrices with one row-major matrix per
// configuration (column b of the (rows * cols) x batch matrix): matrix(), inverse(),
// getInverseOperationalSpaceInertiaMatrix(), getOperationalSpaceInertiaMatrix(),
// getInverseMassMatrix(), getJMinv().
class ContactCholeskyDecomposition {
 public:
  ContactCholeskyDecomposition(const Model& m, const std::vector<RigidConstraintModel>& contact_models)
      : nv_(m.nv), num_contacts_(static_cast<int>(contact_models.size())) {
    for (const auto& c : contact_models) nc_ += c.size();
  }
  void compute(const Model& m, Data& data, const std::vector<RigidConstraintModel>& contact_models,
               const std::vector<RigidConstraintData>& contact_datas, double mu = 0.0) {
    if (contact_models.size() != contact_datas.size())
      throw std::invalid_argument("The contact models and data do not have the same vector size.");
    if (data.q_crba.cols() == 0 && data.q_crba.rows() == 0)
      throw std::invalid_argument("compute reads the configurations of crba(model, data, q): call it first");
    if (!data.constraints || !data.constraints->same(contact_models)) initConstraintDynamics(m, data, contact_models);
    const long B = data.q_crba.cols();
    nc_ = data.constraints->dim();
    num_contacts_ = static_cast<int>(contact_models.size());
    const long n = nc_ + nv_;
    kkt_.resize(n * n, B);
    inverse_.resize(n * n, B);
    osim_inverse_.resize(static_cast<long>(nc_) * nc_, B);
    osim_.resize(static_cast<long>(nc_) * nc_, B);
    minv_.resize(static_cast<long>(nv_) * nv_, B);
    jminv_.resize(static_cast<long>(nc_) * nv_, B);
    const bool c = nc_ > 0;
    check(gb_contact_cholesky(m.get(), data.precision, data.constraints->get(), mu, GB_LAYOUT_INSTANCE, B,
                              data.q_crba.data(), kkt_.data(), inverse_.data(), c ? osim_inverse_.data() : nullptr,
                              c ? osim_.data() : nullptr, minv_.data(), c ? jminv_.data() : nullptr, data.stream));
  }
  int size() const { return nc_ + nv_; }
  int constraintDim() const { return nc_; }
  int numContacts() const { return num_contacts_; }
  const DeviceMatrix& matrix() const { return kkt_; }
  const DeviceMatrix& inverse() const { return inverse_; }
  const DeviceMatrix& getInverseOperationalSpaceInertiaMatrix() const { return osim_inverse_; }
  const DeviceMatrix& getOperationalSpaceInertiaMatrix() const { return osim_; }
  const DeviceMatrix& getInverseMassMatrix() const { return minv_; }
  const DeviceMatrix& getJMinv() const { return jminv_; }

 private:
  int nv_ = 0, nc_ = 0, num_contacts_ = 0;
  DeviceMatrix kkt_, inverse_, osim_inverse_, osim_, minv_, jminv_;
};

// Throws std::runtime_error when the model's kernels recorded a numeric failure
// (gb_numeric_status: a pivot that was not > 0, or a non-finite output); clears the record.
inline void checkNumeric(const Model& m) {
  unsigned int flags = 0;
  check(gb_numeric_status(m.get(), &flags, 1));
}

}  // namespace pinocchio_gb300

#endif  // PINOCCHIO_GB300_HPP
