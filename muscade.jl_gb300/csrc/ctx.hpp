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
  double* cdata = nullptr;  // [nfield][nele] kernel constants (structure of arrays)
  int32_t nfield = 0;
  int64_t tval_base = -1;   // offset in the time-value vector (loads, constraints)
  std::vector<int64_t> h_indexX;  // host copy (1-based) for asm queries
};

struct Solver;  // linear solver state (solver.cu)

}  // namespace mgpu

struct mgpu_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  int64_t nX = 0, nU = 0, ntval = 0;
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
  mgpu::Solver* solver = nullptr;
};

namespace mgpu {
// launches one complete assembly on ctx->stream from the resident state;
// ev_groups (optional) receives an event after each element type's kernel
int launch_assembly(mgpu_ctx* c, int mission, double t, const mgpu_newmark* nm, cudaEvent_t* ev_groups);
int set_err(mgpu_ctx* c, int code, const std::string& msg);
int check_nan(mgpu_ctx* c);
}  // namespace mgpu

#define MG_CUDA(call)                                                                    \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return mgpu::set_err(c, MGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
