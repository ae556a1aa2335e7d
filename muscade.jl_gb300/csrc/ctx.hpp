// Device context shared by the assembly and solver translation units.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/muscade_gpu.h"
#include "pattern.hpp"

namespace mgpu {

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
};

struct DevGroup {
  int32_t kind = 0, nX = 0, nU = 0, ndata = 0;
  int64_t nele = 0;
  int32_t* idx = nullptr;   // [nX][nele] 0-based X dofs (entry-major)
  int32_t* uidx = nullptr;  // [nU][nele] 0-based U dofs
  int32_t* aidx = nullptr;  // [nele] 0-based A-dof (EI scale) of each beam, or nullptr
  std::vector<int64_t> h_indexA;  // host copy (1-based)
  double* cdata = nullptr;  // [nfield][nele] kernel constants (structure of arrays)
  int32_t nfield = 0;
  int64_t tval_base = -1;   // offset in the time-value vector (loads, constraints, cost targets)
  int32_t maxder = 0;       // DOFCOST: highest time derivative a cost reads
  bool distinct = true;     // cost groups: no two elements write the same gradient entry
  std::vector<int64_t> h_indexX;  // host copy (1-based) for asm queries
  std::vector<double> h_edata;    // EULERBEAM3D: the element records as given (for mgpu_beam_results)
};

// element kinds with one time value per element (F(t), c(t) or the cost target y(t))
inline bool has_tval(int kind) {
  return kind == MGPU_DOFLOAD || kind == MGPU_DOFCONSTRAINT_X || kind == MGPU_DOFCOST || kind == MGPU_SINGLEUDOF;
}

struct Solver;  // linear solver state (solver.cu)

}  // namespace mgpu

struct mgpu_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  int64_t nX = 0, nU = 0, ntval = 0, nA = 0;
  double* Avec = nullptr;   // [nA] A-dof values
  std::vector<mgpu::DevGroup> groups;
  mgpu::Pattern pat;
  // device buffers
  double* kbuf = nullptr;   // element matrices, entry-major per group
  double* rbuf = nullptr;   // element vectors
  uint32_t* mseg = nullptr;
  uint32_t* msrc = nullptr;
  uint32_t* vseg = nullptr;
  uint32_t* vsrc = nullptr;
  double* nzval = nullptr;  // [nnz]
  double* Ll = nullptr;     // [nX]
  double* x = nullptr;      // [3][nX] X, X', X''
  double* u = nullptr;      // [nU]
  double* tv = nullptr;     // [ntval]
  double* ab = nullptr;     // [2][nX] Newmark a, b vectors
  double* scale = nullptr;  // [nX] or nullptr
  int* errflag = nullptr;   // [2]: first NaN element (INT_MAX if none), spare
  double* flush = nullptr;  // L2 flush buffer
  size_t flush_bytes = 0;
  int nXder_resident = 1;
  // host: coordinates of each X-dof's node from the beam and bar elements'
  // geometry (NaN where no element gives one) and the constraint multipliers;
  // the sparse solver's ordering uses them
  std::vector<double> dof_xyz;   // [nX][3]
  std::vector<uint8_t> dof_last;  // [nX] 1 for the multiplier of a DofConstraint
  int elem_block = 128;     // threads per block of the beam and bar kernels (mgpu_autotune)
  int64_t launches = 0;     // kernel launches of the assembly, Newton and multifrontal paths (mgpu_launch_count)
  bool device_pattern = false;  // the pattern and plans were built on the device
  mgpu::Solver* solver = nullptr;
  // constants of the current step, read by the kernels from device memory so
  // that a captured step replays with new values: t, a1, a2, a3, b1, b2, b3
  double* stepc = nullptr;   // [8] device
  double* hstepc = nullptr;  // pinned upload ring [kStepcSlots][8]
  cudaEvent_t stepc_ev[8] = {};
  int stepc_slot = 0;
  // pipelined assembly (mgpu_assemble_async): two slots of device outputs and
  // host input staging; a copy stream returns each slot's outputs while the
  // next slot computes
  cudaStream_t cstream = nullptr;
  double* anz[2] = {nullptr, nullptr};   // [nnz] device outputs per slot
  double* aLl[2] = {nullptr, nullptr};   // [nX]
  int* aerr = nullptr;                   // [2] device NaN flags per slot
  int* haerr = nullptr;                  // [2] pinned host copies
  double* astage[2] = {nullptr, nullptr};  // pinned host staging: x [3nX], u [nU], tvals [ntval]
  cudaEvent_t a_h2d[2] = {}, a_comp[2] = {}, a_d2h[2] = {};
  bool a_used[2] = {false, false};
  int64_t aticket = 0;
};

namespace mgpu {
constexpr int kStepcSlots = 8;
// enqueue the upload of the step constants (t and the Newmark coefficients,
// zero when nm is NULL) to ctx->stepc
int upload_stepc(mgpu_ctx* c, double t, const mgpu_newmark* nm);
// launches one complete assembly on ctx->stream from the resident state and
// step constants; ev_groups (optional) receives an event after each element
// type's kernel.  The matrix is p0 ∂R/∂X + a1 ∂R/∂X' + b1 ∂R/∂X'' with a1, b1
// from the step constants (p0 = 1 in the Newton loops; 0 to assemble the
// damping or mass matrix alone).  Enqueues no copy and no synchronisation
// (capturable).
int launch_assembly(mgpu_ctx* c, int mission, cudaEvent_t* ev_groups, double p0 = 1.0);
// errflag <- INT_MAX on ctx->stream (capturable)
void launch_reset_errflag(mgpu_ctx* c);
int set_err(mgpu_ctx* c, int code, const std::string& msg);
int check_nan(mgpu_ctx* c);
// MGPU_ERR_NAN with the reference's message for an errflag value (MGPU_OK for INT_MAX)
int nan_error(mgpu_ctx* c, int flag);
}  // namespace mgpu

#define MG_CUDA(call)                                                                    \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return mgpu::set_err(c, MGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
