// Library-wide pieces of the C ABI: version, last-error string, device count,
// stream/precision setters, destroy, and the fixed-order residual finalizer.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "common.cuh"

namespace fpie {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }

// One block: thread t sums partials t, t+256, ... in double; the block tree
// then adds the 256 per-thread sums.  Same order on every call.
__global__ void __launch_bounds__(256)
finalize_kernel(const double* __restrict__ parts, int nparts,
                float* __restrict__ err) {
  double a = 0.0, b = 0.0, c = 0.0;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x) {
    a += parts[3 * k + 0];
    b += parts[3 * k + 1];
    c += parts[3 * k + 2];
  }
  block_sum3(a, b, c);
  if (threadIdx.x == 0) {
    err[0] = (float)a;
    err[1] = (float)b;
    err[2] = (float)c;
  }
}

void launch_finalize(const double* parts, int nparts, float* err,
                     cudaStream_t st) {
  finalize_kernel<<<1, 256, 0, st>>>(parts, nparts, err);
}

int stride_blocks(long long total, int threads, int per_sm) {
  static std::mutex mu;
  static int sms[64] = {};
  int dev = 0;
  FPIE_CUDA(cudaGetDevice(&dev));
  FPIE_REQUIRE(dev >= 0 && dev < 64, FPIE_ERR_STATE, "device ordinal out of range");
  int n;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!sms[dev]) FPIE_CUDA(cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev));
    n = sms[dev];
  }
  const long long want = (total + threads - 1) / threads;
  return (int)std::max<long long>(1, std::min<long long>(want, (long long)n * per_sm));
}

cudaMemPool_t scratch_pool() {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  int dev = 0;
  FPIE_CUDA(cudaGetDevice(&dev));
  FPIE_REQUIRE(dev >= 0 && dev < 64, FPIE_ERR_STATE, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(mu);
  if (!pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p = nullptr;
    FPIE_CUDA(cudaMemPoolCreate(&p, &props));
    uint64_t keep = 4ULL << 30;
    FPIE_CUDA(cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep));
    pools[dev] = p;
  }
  return pools[dev];
}

}  // namespace fpie

using namespace fpie;

extern "C" {

int fpie_version(void) { return 100; }

const char* fpie_last_error(void) { return g_last_error.c_str(); }

int fpie_device_count(int* count) {
  return guarded([&] {
    FPIE_REQUIRE(count != nullptr, FPIE_ERR_ARG, "null count pointer");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
      cudaGetLastError();
      n = 0;
    }
    *count = n;
  });
}

int fpie_equ_create(int block_size, fpie_solver** out) {
  return guarded([&] {
    FPIE_REQUIRE(out != nullptr, FPIE_ERR_ARG, "null output pointer");
    *out = reinterpret_cast<fpie_solver*>(new_equ_solver(block_size));
  });
}

int fpie_grid_create(int grid_x, int grid_y, fpie_solver** out) {
  return guarded([&] {
    FPIE_REQUIRE(out != nullptr, FPIE_ERR_ARG, "null output pointer");
    *out = reinterpret_cast<fpie_solver*>(new_grid_solver(grid_x, grid_y));
  });
}

int fpie_destroy(fpie_solver* s) {
  return guarded([&] {
    if (s == nullptr) return;
    Solver* h = reinterpret_cast<Solver*>(s);
    cudaSetDevice(h->device);
    delete h;
  });
}

int fpie_sync(fpie_solver* s) {
  return guarded([&] {
    Solver* h = check_handle(s, 0);
    FPIE_CUDA(cudaStreamSynchronize(h->stream));
    h->check_async();
  });
}

int fpie_set_stream(fpie_solver* s, void* stream) {
  return guarded([&] {
    Solver* h = check_handle(s, 0);
    // NULL is a valid choice: the legacy default stream (torch's default).
    h->stream = reinterpret_cast<cudaStream_t>(stream);
  });
}

int fpie_launch_count(fpie_solver* s, long long* count) {
  return guarded([&] {
    Solver* h = check_handle(s, 0);
    FPIE_REQUIRE(count != nullptr, FPIE_ERR_ARG, "null count pointer");
    *count = h->launches;
  });
}

}  // extern "C"
