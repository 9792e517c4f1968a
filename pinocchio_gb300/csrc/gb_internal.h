// Internal host-side declarations shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/pinocchio_gb300.h"
#include "gb_model_build.h"

struct gb_pool {
  const gb_model* model = nullptr;
  long size = 0;
  int precision = GB_FP64;
  cudaStream_t stream = nullptr;
  double* d_buf = nullptr;  // device staging for the *_in_parallel calls
  size_t d_bytes = 0;
};

namespace gbi {

// One rigid constraint model as the kernels read it (gb_constraint_set): the joints of the
// internal tree and the placements relative to their (folded) frames; `row` is the first
// constraint row, `gains` whether any Baumgarte gain is non-zero.
struct ConstraintDev {
  int type, frame, j1, j2, row, gains, pad0, pad1;
  double P1[12], P2[12], des[6], Kp[6], Kd[6];
};

}  // namespace gbi

struct gb_constraint_set {
  const gb_model* model = nullptr;
  int n = 0, nc = 0;
  std::vector<gbi::ConstraintDev> host;
  // per constraint and dof: 0 no column, 1 joint 1's side only, 2 joint 2's side only, 3 both
  std::vector<signed char> sparsity;
  void* d_mem = nullptr;  // the table, then the sparsity codes
};

namespace gbi {

int set_error(int code, const std::string& msg);
int cuda_error(cudaError_t e, const char* where);

// per-instance strides of one batch array
struct Arr {
  const double* p;
  long is;  // instance stride
  long es;  // element stride
};
inline Arr arr(const double* p, int layout, long batch, long n) {
  return layout == GB_LAYOUT_SOA ? Arr{p, 1, batch} : Arr{p, n, 1};
}

// check_common also refuses models with mimic joints (the functions that take them call
// check_common_mimic and the *_mimic launches below)
int check_common(const gb_model* m, int precision, int layout, long batch);
int check_common_mimic(const gb_model* m, int precision, int layout, long batch);
int check_ptr(const void* p, const char* name);


// launches (gb_kernels.cu / gb_derivs.cu)
int launch_rnea(const gb_model* m, int precision, long B, Arr q, Arr v, Arr a, Arr tau, cudaStream_t st);
int launch_aba(const gb_model* m, int precision, long B, Arr q, Arr v, Arr tau, Arr ddq, cudaStream_t st);
// with external forces (njoints x 6 per configuration): one thread per configuration
int launch_rnea_fext(const gb_model* m, int precision, long B, Arr q, Arr v, Arr a, Arr fext, Arr tau, cudaStream_t st);
int launch_aba_fext(const gb_model* m, int precision, long B, Arr q, Arr v, Arr tau, Arr fext, Arr ddq, cudaStream_t st);
// warp-per-instance layout (gb_warp.cu)
int launch_rnea_warp(const gb_model* M, int precision, long B, Arr q, Arr v, Arr a, Arr tau, cudaStream_t st);
int launch_aba_warp(const gb_model* M, int precision, long B, Arr q, Arr v, Arr tau, Arr ddq, cudaStream_t st);
// lane-per-branch layout (gb_warp.cu)
int launch_rnea_branch(const gb_model* M, int precision, long B, Arr q, Arr v, Arr a, Arr tau, cudaStream_t st);
int launch_aba_branch(const gb_model* M, int precision, long B, Arr q, Arr v, Arr tau, Arr ddq, cudaStream_t st);
int launch_crba(const gb_model* m, int precision, bool symmetric, long B, Arr q, Arr M, Arr U, Arr D, cudaStream_t st);
// forwardDynamics / impulseDynamics with a given constraint Jacobian (gb_contact.cu)
int launch_contact(const gb_model* m, int precision, bool impulse, long B, int nc, Arr q, Arr v, Arr x, Arr J,
                   Arr gamma, double r_coeff, double inv_damping, Arr out, Arr lam, cudaStream_t st);
int launch_kkt_inverse(const gb_model* m, long B, int nc, Arr q, Arr J, double inv_damping, Arr K, cudaStream_t st);
int check_gravity(const gb_model* M);  // GB_ERR_GRAVITY when the gravity has an angular part
int launch_rnea_derivs_fext(const gb_model* M, int precision, long B, Arr q, Arr v, Arr a, Arr fext, Arr dq, Arr dv,
                            Arr Mo, cudaStream_t st);
int launch_constraint_derivs(const gb_model* M, int precision, long B, const gb_constraint_set* set,
                             const gb_proximal_settings& s, Arr q, Arr v, Arr tau, Arr ddq, Arr lam, Arr ddq_dq,
                             Arr ddq_dv, Arr ddq_dtau, Arr dl_dq, Arr dl_dv, Arr dl_dtau, int* iters, cudaStream_t st);
int launch_constraint(const gb_model* M, int precision, long B, const gb_constraint_set* set,
                      const gb_proximal_settings& s, Arr q, Arr v, Arr tau, Arr ddq, Arr lam, int* iters,
                      double* residuals, cudaStream_t st,
                      double* U_keep = nullptr, double* D_keep = nullptr);
int launch_contact_cholesky(const gb_model* M, long B, const gb_constraint_set* set, double mu, Arr q, Arr kkt,
                            Arr kinv, Arr oinv, Arr osim, Arr minv, Arr jminv, cudaStream_t st);
int launch_integrate(const gb_model* m, long B, Arr q, Arr v, Arr qo, cudaStream_t st);
int launch_fk(const gb_model* m, int precision, long B, Arr q, Arr v, Arr a, Arr oMi, Arr vo, Arr ao, cudaStream_t st);
int launch_jacobians(const gb_model* m, int precision, long B, Arr q, Arr J, cudaStream_t st);
// models with mimic joints (gb_mimic.cu): the caller's arrays mapped to and from the extended tree
int launch_rnea_mimic(const gb_model* M, int precision, long B, Arr q, Arr v, Arr a, Arr tau, cudaStream_t st);
int launch_rnea_fext_mimic(const gb_model* M, int precision, long B, Arr q, Arr v, Arr a, Arr fext, Arr tau,
                           cudaStream_t st);
int launch_crba_mimic(const gb_model* M, int precision, bool symmetric, long B, Arr q, Arr Mout, cudaStream_t st);
int launch_fk_mimic(const gb_model* M, int precision, long B, Arr q, Arr v, Arr a, Arr oMi, Arr vout, Arr aout,
                    cudaStream_t st);
int launch_jacobians_mimic(const gb_model* M, int precision, long B, Arr q, Arr J, cudaStream_t st);
int launch_integrate_mimic(const gb_model* M, long B, Arr q, Arr v, Arr qout, cudaStream_t st);
size_t aba_derivs_workspace_bytes(const gb_model* M, int precision, long B);
// per-model launch preparation at creation (gb_derivs.cu)
int prepare_model_launches(gb_model* M);
// device scratch from the stream-ordered pool, and the SOA -> instance transpose (gb_util.cu):
// src holds n elements x B configurations ([element][configuration]), dst an instance-layout array
int scratch_alloc(void** p, size_t bytes, cudaStream_t st);
void scratch_free(void* p, cudaStream_t st);
int launch_soa_to_instance(const double* src, long B, long n, Arr dst, cudaStream_t st);
// batches from which the matrix outputs of the per-thread kernels go through an SOA scratch
constexpr long kSoaStagingMin = 1024;
int launch_aba_derivs_on_workspace(const gb_model* M, int precision, long B, Arr q, Arr v, Arr tau, Arr dq, Arr dv,
                                   Arr Minv, Arr ddq, void* ws, cudaStream_t st);

}  // namespace gbi
