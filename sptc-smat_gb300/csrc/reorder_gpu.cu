// reorder_gpu.cu — candidate distances of the Keeper row grouping on a GPU.
//
// The reference's IterativeBlockingKeeper (preprocess/src/general/blocking.cpp:431-547)
// measures, for each seed row, every later row against the seed group's
// block-column pattern with JaccardDistanceGroup (blocking.cpp:904-975) and
// merges the first one within tau. reorder.cpp keeps that sequential commit
// on the host; this file measures a whole chunk of candidates at once, one
// thread per candidate row, and returns the distances.
//
// Each thread walks the pattern P (na block ids, group size g; in shared
// memory when it fits) and its candidate row R (nb ids) the way the
// reference's distance function does: an id taken from P alone adds 1 to
// count, one taken from R alone adds g, equal ids add nothing, and the tails
// are added at the end; then
//   dist = (float)(2 count / (double)(na g + nb + count)),
// 0 when both lists are empty and 1 when exactly one is. The walk is the
// same step for step as the host's (also for lists that are not sorted),
// every term is an integer below 2^53, so the double quotient is the
// correctly rounded one on both sides and the float cast matches the host's
// bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "smat_internal.h"

namespace smat {
namespace dev {

constexpr int kPatternSmem = 8192;  // pattern ids staged in shared memory (32 KB)

__global__ void __launch_bounds__(256) keeper_dist_kernel(const int32_t* __restrict__ runs,
                                                          const int64_t* __restrict__ run_ptr,
                                                          const int32_t* __restrict__ pattern, int64_t np,
                                                          int64_t g, int64_t j0, int64_t j1,
                                                          float* __restrict__ out) {
  __shared__ int32_t sp[kPatternSmem];
  const bool in_smem = np <= kPatternSmem;
  if (in_smem)
    for (int64_t i = threadIdx.x; i < np; i += blockDim.x) sp[i] = pattern[i];
  __syncthreads();
  const int32_t* P = in_smem ? sp : pattern;
  for (int64_t j = j0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < j1; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b0 = run_ptr[j], nb = run_ptr[j + 1] - b0;
    float d;
    if (np == 0 && nb == 0) {
      d = 0.0f;
    } else if (np == 0 || nb == 0) {
      d = 1.0f;
    } else {
      const int32_t* R = runs + b0;
      int64_t i = 0, k = 0, count = 0;
      while (i < np && k < nb) {
        const int32_t a = P[i], b = R[k];
        if (a < b) {
          count += 1;
          ++i;
        } else if (a > b) {
          count += g;
          ++k;
        } else {
          ++i;
          ++k;
        }
      }
      count += (np - i) + (nb - k) * g;
      d = (float)((2.0 * (double)count) / (double)(np * g + nb + count));
    }
    out[j - j0] = d;
  }
}

}  // namespace dev

namespace {

class CudaKeeper final : public KeeperDevice {
 public:
  explicit CudaKeeper(int device) : device_(device) {}
  ~CudaKeeper() override {
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(device_);
    cudaFree(d_runs_);
    cudaFree(d_ptr_);
    cudaFree(d_pat_);
    cudaFree(d_out_);
    cudaFreeHost(h_out_);
    if (stream_) cudaStreamDestroy(stream_);
    if (prev >= 0) cudaSetDevice(prev);
  }

  bool init(const std::vector<int64_t>& runs, const std::vector<int64_t>& run_ptr) override {
    if (!set_device()) return false;
    if (!ok(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream")) return false;
    if (!ok(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, device_), "SM count")) return false;
    std::vector<int32_t> r32(runs.size());
    for (size_t i = 0; i < runs.size(); i++) {
      if (runs[i] < 0 || runs[i] > INT32_MAX) return bad("block-column id out of 32-bit range");
      r32[i] = (int32_t)runs[i];
    }
    rows_ = (int64_t)run_ptr.size() - 1;
    const size_t rb = std::max<size_t>(r32.size(), 1) * sizeof(int32_t);
    return ok(cudaMalloc(&d_runs_, rb), "cudaMalloc runs") &&
           ok(cudaMalloc(&d_ptr_, run_ptr.size() * sizeof(int64_t)), "cudaMalloc run_ptr") &&
           (r32.empty() || ok(cudaMemcpy(d_runs_, r32.data(), r32.size() * sizeof(int32_t), cudaMemcpyHostToDevice),
                              "copy runs")) &&
           ok(cudaMemcpy(d_ptr_, run_ptr.data(), run_ptr.size() * sizeof(int64_t), cudaMemcpyHostToDevice),
              "copy run_ptr");
  }

  bool fill(const int64_t* pattern, int64_t np, int64_t g, int64_t j0, int64_t j1, float* out) override {
    if (j1 <= j0) return true;
    if (j0 < 0 || j1 > rows_) return bad("candidate range outside the matrix");
    if (!set_device()) return false;
    const int64_t n = j1 - j0;
    if (n > out_cap_) {
      cudaFree(d_out_);
      cudaFreeHost(h_out_);
      d_out_ = nullptr;
      h_out_ = nullptr;
      out_cap_ = 0;
      if (!ok(cudaMalloc(&d_out_, (size_t)n * sizeof(float)), "cudaMalloc distances") ||
          !ok(cudaMallocHost(&h_out_, (size_t)n * sizeof(float)), "cudaMallocHost distances"))
        return false;
      out_cap_ = n;
    }
    if (np > pat_cap_) {
      cudaFree(d_pat_);
      d_pat_ = nullptr;
      pat_cap_ = 0;
      if (!ok(cudaMalloc(&d_pat_, (size_t)np * sizeof(int32_t)), "cudaMalloc pattern")) return false;
      pat_cap_ = np;
    }
    // the pattern changes after every merge: send it with each chunk
    pat32_.resize((size_t)np);
    for (int64_t i = 0; i < np; i++) pat32_[i] = (int32_t)pattern[i];
    if (np > 0 && !ok(cudaMemcpyAsync(d_pat_, pat32_.data(), (size_t)np * sizeof(int32_t), cudaMemcpyHostToDevice,
                                      stream_),
                      "copy pattern"))
      return false;
    const int threads = 256;
    const int64_t blocks = std::min<int64_t>((n + threads - 1) / threads, (int64_t)sms_ * 8);
    dev::keeper_dist_kernel<<<(unsigned)blocks, threads, 0, stream_>>>(d_runs_, d_ptr_, d_pat_, np, g, j0, j1, d_out_);
    if (!ok(cudaGetLastError(), "distance kernel launch") ||
        !ok(cudaMemcpyAsync(h_out_, d_out_, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, stream_),
            "copy distances") ||
        !ok(cudaStreamSynchronize(stream_), "distance kernel"))
      return false;
    std::copy(h_out_, h_out_ + n, out);
    return true;
  }

  const char* error() const override { return err_.c_str(); }

 private:
  bool set_device() { return ok(cudaSetDevice(device_), "cudaSetDevice"); }
  bool ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    err_ = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
  }
  bool bad(const char* why) {
    err_ = why;
    return false;
  }

  int device_;
  int sms_ = 1;
  int64_t rows_ = 0;
  cudaStream_t stream_ = nullptr;
  int32_t* d_runs_ = nullptr;
  int64_t* d_ptr_ = nullptr;
  int32_t* d_pat_ = nullptr;
  int64_t pat_cap_ = 0;
  float* d_out_ = nullptr;
  float* h_out_ = nullptr;
  int64_t out_cap_ = 0;
  std::vector<int32_t> pat32_;
  std::string err_;
};

}  // namespace

KeeperDevice* make_keeper_device(int device) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return nullptr;
  return new CudaKeeper(device);
}

}  // namespace smat
