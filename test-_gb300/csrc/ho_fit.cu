// The GPU modal fitter: the scene loader's tensor-product fit of each
// element's nodal geometry (FP64 values on GLL nodes) into Modified-A
// coefficients (FEM-AABB/xml_fld_math.cpp:379-483, TensorModalFit3D), for
// many elements at once.
//
// Jobs are gathered in pinned host memory; a batch (up to kFitBatchBytes of
// nodal values) is copied to the device and fitted by one CTA per element:
// the element's component block sits in shared memory and the three 1-D
// inverse-Vandermonde passes (r, then s, then t) run with one thread per
// output value, summing in the host fitter's order; the FP32 coefficients come
// back and are scattered to each job's destination.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "ho_host.h"

namespace ho {

namespace {

constexpr int kFitThreads = 256;
constexpr size_t kFitBatchBytes = size_t(64) << 20;  // nodal values per batch
constexpr int kVinvStride = kMaxModes * kMaxModes;  // one n x n inverse per n

struct FitJob {
  int64_t src;   // first nodal value (doubles)
  int64_t dst;   // first coefficient (floats) in the batch's output
  int nx, ny, nz, comps;
};

__global__ void __launch_bounds__(kFitThreads) fit_kernel(const FitJob* __restrict__ jobs,
                                                          const double* __restrict__ src,
                                                          const double* __restrict__ vinv, float* __restrict__ dst) {
  __shared__ double A[kMaxModes * kMaxModes * kMaxModes];
  __shared__ double B[kMaxModes * kMaxModes * kMaxModes];
  const FitJob jb = jobs[blockIdx.x];
  const int nx = jb.nx, ny = jb.ny, nz = jb.nz;
  const int S = nx * ny * nz;
  const double* vr = vinv + nx * kVinvStride;
  const double* vs = vinv + ny * kVinvStride;
  const double* vt = vinv + nz * kVinvStride;
  for (int c = 0; c < jb.comps; ++c) {
    const double* a = src + jb.src + static_cast<int64_t>(c) * S;
    for (int q = threadIdx.x; q < S; q += blockDim.x) A[q] = a[q];
    __syncthreads();
    for (int q = threadIdx.x; q < S; q += blockDim.x) {  // r: B[m,j,k] = sum_i vr[m][i] A[i,j,k]
      const int m = q % nx, jk = q / nx;
      double s = 0;
      for (int i = 0; i < nx; ++i) s += vr[m * nx + i] * A[jk * nx + i];
      B[q] = s;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < S; q += blockDim.x) {  // s: A[i,m,k] = sum_j vs[m][j] B[i,j,k]
      const int i = q % nx, m = (q / nx) % ny, k = q / (nx * ny);
      double s = 0;
      for (int j = 0; j < ny; ++j) s += vs[m * ny + j] * B[(k * ny + j) * nx + i];
      A[q] = s;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < S; q += blockDim.x) {  // t: out[i,j,m] = sum_k vt[m][k] A[i,j,k]
      const int ij = q % (nx * ny), m = q / (nx * ny);
      double s = 0;
      for (int k = 0; k < nz; ++k) s += vt[m * nz + k] * A[k * nx * ny + ij];
      dst[jb.dst + static_cast<int64_t>(c) * S + q] = static_cast<float>(s);
    }
    __syncthreads();
  }
}

class GpuFitter final : public ModalFitter {
 public:
  explicit GpuFitter(int device) : device_(device) {}
  ~GpuFitter() override {
    cudaFreeHost(h_src_);
    cudaFreeHost(h_dst_);
    cudaFree(d_src_);
    cudaFree(d_dst_);
    cudaFree(d_jobs_);
    cudaFree(d_vinv_);
    if (stream_) cudaStreamDestroy(stream_);
  }

  bool add(const double* nodal, int comps, int nx, int ny, int nz, std::vector<float>* dst, int64_t dst_off) override {
    if (!ok_ || !init()) return false;
    for (int n : {nx, ny, nz})
      if (n < 1 || n > kMaxModes) return fail("modes outside 1..9");
    const int64_t vals = static_cast<int64_t>(comps) * nx * ny * nz;
    if (n_src_ + vals > cap_src_ && !flush()) return false;
    if (vals > cap_src_) return fail("element larger than a batch");
    std::memcpy(h_src_ + n_src_, nodal, static_cast<size_t>(vals) * sizeof(double));
    FitJob j;
    j.src = n_src_;
    j.dst = n_src_;  // the output has one float per nodal value, at the same position
    j.nx = nx;
    j.ny = ny;
    j.nz = nz;
    j.comps = comps;
    jobs_.push_back(j);
    where_.push_back({dst, dst_off});
    n_src_ += vals;
    return true;
  }

  bool finish() override { return ok_ && (jobs_.empty() || flush()); }
  const char* error() const override { return err_.c_str(); }

 private:
  struct Where {
    std::vector<float>* dst;
    int64_t off;
  };

  bool fail(const std::string& m) {
    ok_ = false;
    err_ = "GPU modal fit: " + m;
    return false;
  }
  bool cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    cudaGetLastError();
    return fail(std::string(what) + ": " + cudaGetErrorString(e));
  }

  bool init() {
    if (h_src_) return true;
    cap_src_ = static_cast<int64_t>(kFitBatchBytes / sizeof(double));
    if (!cuda(cudaSetDevice(device_), "cudaSetDevice")) return false;
    if (!cuda(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate")) return false;
    if (!cuda(cudaMallocHost(&h_src_, cap_src_ * sizeof(double)), "cudaMallocHost")) return false;
    if (!cuda(cudaMallocHost(&h_dst_, cap_src_ * sizeof(float)), "cudaMallocHost")) return false;
    if (!cuda(cudaMalloc(&d_src_, cap_src_ * sizeof(double)), "cudaMalloc")) return false;
    if (!cuda(cudaMalloc(&d_dst_, cap_src_ * sizeof(float)), "cudaMalloc")) return false;
    // inverse Vandermonde matrices at the GLL nodes for n = 1..9 (row-major n x n)
    std::vector<double> vinv(static_cast<size_t>(kMaxModes + 1) * kVinvStride, 0.0);
    for (int n = 1; n <= kMaxModes; ++n) {
      std::vector<double> inv;
      if (!modal_vandermonde_inverse(gll_nodes(n), inv)) return fail("Vandermonde matrix not invertible");
      std::copy(inv.begin(), inv.end(), vinv.begin() + static_cast<size_t>(n) * kVinvStride);
    }
    if (!cuda(cudaMalloc(&d_vinv_, vinv.size() * sizeof(double)), "cudaMalloc")) return false;
    return cuda(cudaMemcpy(d_vinv_, vinv.data(), vinv.size() * sizeof(double), cudaMemcpyHostToDevice), "copy");
  }

  bool flush() {
    if (jobs_.empty()) return true;
    const size_t nj = jobs_.size();
    if (nj > jobs_cap_) {
      cudaFree(d_jobs_);
      d_jobs_ = nullptr;
      if (!cuda(cudaMalloc(&d_jobs_, nj * sizeof(FitJob)), "cudaMalloc")) return false;
      jobs_cap_ = nj;
    }
    const size_t bytes = static_cast<size_t>(n_src_) * sizeof(double);
    if (!cuda(cudaMemcpyAsync(d_src_, h_src_, bytes, cudaMemcpyHostToDevice, stream_), "copy nodal values") ||
        !cuda(cudaMemcpyAsync(d_jobs_, jobs_.data(), nj * sizeof(FitJob), cudaMemcpyHostToDevice, stream_),
              "copy jobs"))
      return false;
    fit_kernel<<<static_cast<unsigned>(nj), kFitThreads, 0, stream_>>>(d_jobs_, d_src_, d_vinv_, d_dst_);
    if (!cuda(cudaGetLastError(), "fit kernel") ||
        !cuda(cudaMemcpyAsync(h_dst_, d_dst_, static_cast<size_t>(n_src_) * sizeof(float), cudaMemcpyDeviceToHost,
                              stream_),
              "copy coefficients") ||
        !cuda(cudaStreamSynchronize(stream_), "fit"))
      return false;
    for (size_t q = 0; q < nj; ++q) {
      const FitJob& j = jobs_[q];
      const int64_t vals = static_cast<int64_t>(j.comps) * j.nx * j.ny * j.nz;
      std::memcpy(where_[q].dst->data() + where_[q].off, h_dst_ + j.dst, static_cast<size_t>(vals) * sizeof(float));
    }
    jobs_.clear();
    where_.clear();
    n_src_ = 0;
    return true;
  }

  int device_;
  bool ok_ = true;
  std::string err_ = "GPU modal fit failed";
  cudaStream_t stream_ = nullptr;
  double* h_src_ = nullptr;
  float* h_dst_ = nullptr;
  double* d_src_ = nullptr;
  float* d_dst_ = nullptr;
  double* d_vinv_ = nullptr;
  FitJob* d_jobs_ = nullptr;
  size_t jobs_cap_ = 0;
  int64_t cap_src_ = 0, n_src_ = 0;
  std::vector<FitJob> jobs_;
  std::vector<Where> where_;
};

}  // namespace

std::unique_ptr<ModalFitter> make_gpu_fitter(int device) { return std::make_unique<GpuFitter>(device); }

}  // namespace ho
