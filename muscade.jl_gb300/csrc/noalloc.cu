// Beam assembly for callers that cannot allocate device memory.
//
// Some host programs cannot call cudaMalloc at the point where they need an
// assembly: code running inside a captured CUDA graph, a real-time loop whose
// memory was fixed up front, or a process whose device memory belongs to
// another runtime's pool.  mgpu_assemble_beams_noalloc serves them: the caller
// passes every input and output as device memory it already owns, and the only
// scratch the computation needs -- the per-element residuals and tangents
// before they are summed -- lives in a fixed file-scope device array,
// g_noalloc_scratch, sized for MGPU_NOALLOC_MAX_BEAMS elements.  Every GPU that
// loads this library holds that array until the process exits.
//
// The summation follows the reference's assembly order (element by element,
// entries through the asm maps), so for beams without U- or A-dofs and with
// unit dof scales the results equal those of mgpu_assemble for the same
// beams.  U-dof loads, A-dof EI scales and dis.scaleX are not applied, and no
// NaN check is made: a NaN in an element reaches Lλ / nzval through the sums.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/muscade_gpu.h"
#include "beam_const.hpp"

namespace {

constexpr int64_t kMaxBeams = MGPU_NOALLOC_MAX_BEAMS;
constexpr int kEntries = 144 + 12;  // element matrix and vector entries
constexpr int kRows = kEntries + 1;  // and one row of repeated-dof flags

// Shared scratch of every call (and every stream) on a device.
static __device__ __align__(256) double g_noalloc_scratch[kMaxBeams * kRows];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_addr[kMaxDevices] = {nullptr};

// Element kernel: static (SweepX{0}) residual and tangent of each beam, written
// to scratch entry-major: matrix entry k of element e at k*nele+e, vector entry
// i at (144+i)*nele+e, and at (156)*nele+e 1.0 when the element lists one dof
// twice (its entries may then add into the same place), else 0.0.
__global__ void noalloc_beam_kernel(int64_t nele, const double* __restrict__ fields,
                                    const int64_t* __restrict__ indexX, const double* __restrict__ x,
                                    double* __restrict__ scratch) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= nele) return;
  mgpu::BeamConst bc;
  mgpu::beam_const_from_fields(fields + e * 69, bc);
  int64_t dof[12];
  for (int i = 0; i < 12; ++i) dof[i] = indexX[e * 12 + i];
  bool repeated = false;
  for (int i = 0; i < 12; ++i)
    for (int j = i + 1; j < 12; ++j) repeated |= dof[i] == dof[j];
  scratch[int64_t(kEntries) * nele + e] = repeated ? 1.0 : 0.0;
  double X0[12];
  for (int i = 0; i < 12; ++i) X0[i] = x[dof[i] - 1];
  double R[12], K[144];
  mgpu::beam_element<false>(bc, X0, X0, X0, nullptr, mgpu::Perturb{1.0, 0.0, 0.0}, nullptr, nullptr, R, K, nullptr,
                            nullptr);
  for (int k = 0; k < 144; ++k) scratch[k * nele + e] = K[k];
  for (int i = 0; i < 12; ++i) scratch[(144 + i) * nele + e] = R[i];
}

// One block adds the elements in order (add_value!/add_∂!, src/Assemble.jl:559-608);
// the entries of one element go in parallel unless the element repeats a dof
// (flag row of the element kernel), in which case one thread adds them in the
// reference's entry order.
__global__ void noalloc_accumulate(int64_t nele, const int64_t* __restrict__ asm1, const int64_t* __restrict__ asm2,
                                   const double* __restrict__ scratch, double* __restrict__ Ll,
                                   double* __restrict__ nzval) {
  for (int64_t e = 0; e < nele; ++e) {
    const bool repeated = scratch[int64_t(kEntries) * nele + e] != 0.0;  // uniform over the block
    if (!repeated) {
      for (int k = threadIdx.x; k < kEntries; k += blockDim.x) {
        if (k < 144) {
          const int64_t q = asm2[e * 144 + k];
          if (q != 0) nzval[q - 1] += scratch[k * nele + e];
        } else {
          const int64_t q = asm1[e * 12 + (k - 144)];
          if (q != 0) Ll[q - 1] += scratch[k * nele + e];
        }
      }
    } else if (threadIdx.x == 0) {
      for (int k = 0; k < kEntries; ++k) {
        if (k < 144) {
          const int64_t q = asm2[e * 144 + k];
          if (q != 0) nzval[q - 1] += scratch[k * nele + e];
        } else {
          const int64_t q = asm1[e * 12 + (k - 144)];
          if (q != 0) Ll[q - 1] += scratch[k * nele + e];
        }
      }
    }
    __syncthreads();
  }
}

// Address of the scratch array on the current device, looked up once per device.
int scratch_address(int device, double** out) {
  if (device < 0 || device >= kMaxDevices) return MGPU_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) return MGPU_ERR_CUDA;
    g_scratch_addr[device] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[device];
  return MGPU_OK;
}

}  // namespace

extern "C" int mgpu_assemble_beams_noalloc(int64_t nele, int64_t nX, int64_t nnz, const double* fields,
                                           const int64_t* indexX, const int64_t* asm1, const int64_t* asm2,
                                           const double* x, double* Ll, double* nzval, void* stream) {
  if (nele < 0 || nX < 0 || nnz < 0 || (nele > 0 && (!fields || !indexX || !asm1 || !asm2 || !x)) ||
      (nX > 0 && !Ll) || (nnz > 0 && !nzval))
    return MGPU_ERR_ARG;
  if (nele > kMaxBeams) return MGPU_ERR_SIZE;
  // an error left by the caller's earlier CUDA work on this thread is reported
  // as it stands, before anything is enqueued (it is not cleared)
  if (cudaPeekAtLastError() != cudaSuccess) return MGPU_ERR_CUDA;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return MGPU_ERR_CUDA;
  double* scratch = nullptr;
  const int rc = scratch_address(device, &scratch);
  if (rc != MGPU_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // Lλ and Lλx.nzval start from zero, like zero!(out) (src/Assemble.jl:534-546)
  if (nX > 0 && cudaMemsetAsync(Ll, 0, size_t(nX) * sizeof(double), st) != cudaSuccess) return MGPU_ERR_CUDA;
  if (nnz > 0 && cudaMemsetAsync(nzval, 0, size_t(nnz) * sizeof(double), st) != cudaSuccess) return MGPU_ERR_CUDA;
  if (nele > 0) {
    noalloc_beam_kernel<<<unsigned((nele + 63) / 64), 64, 0, st>>>(nele, fields, indexX, x, scratch);
    if (cudaGetLastError() != cudaSuccess) return MGPU_ERR_CUDA;
    noalloc_accumulate<<<1, 256, 0, st>>>(nele, asm1, asm2, scratch, Ll, nzval);
  }
  return cudaGetLastError() == cudaSuccess ? MGPU_OK : MGPU_ERR_CUDA;
}
