/* ORACLE (benchmark/test infrastructure only): the host side of the
 * reference's own CUDA solvers, so that the kernels its sources compile to
 * run unchanged on this GPU beside the GB300 backend.
 *
 * oracle/build_ref.sh compiles the reference's fpie/core/cuda/grid.cu and
 * fpie/core/cuda/equ.cu (device code, -cubin for sm_103a) into
 * oracle/_ref/cuda/.  This file loads those modules with the CUDA driver API
 * and restates the reference's host step loops:
 *   - CudaGridSolver::step (fpie/core/cuda/grid.cu:133-153): clear err,
 *     `iteration` launches of iter_grid_kernel over blocks of grid_x x grid_y
 *     threads covering the N x M crop, device synchronize, then
 *     copy_img_grid_kernel and error_grid_kernel, synchronize, copy err and
 *     the image back;
 *   - CudaEquSolver::step (fpie/core/cuda/equ.cu:189-211): the same with
 *     iter_equ_kernel over unknowns 1..N-1 in 1-D blocks of block_size, then
 *     copy_X_equ_kernel, error_equ_kernel and error_sum_equ_kernel.
 * The device buffers (the reference's post_reset allocations,
 * fpie/core/cuda/grid.cu:33-52, equ.cu:56-74) are passed in by the caller.
 * Every call returns a CUresult (0 = success).  Kernels run on `stream`. */
#include <cuda.h>
#include <stddef.h>

static CUmodule g_grid_mod, g_equ_mod;
static CUfunction f_iter_grid, f_copy_grid, f_err_grid;
static CUfunction f_iter_equ, f_copy_equ, f_err_equ, f_errsum_equ;

#define CHECK(x)                   \
  do {                             \
    CUresult r_ = (x);             \
    if (r_ != CUDA_SUCCESS) return r_; \
  } while (0)

/* Kernel names as the reference declares them (C++ linkage). */
int refcuda_load(const char* grid_cubin, const char* equ_cubin) {
  CUcontext ctx = NULL;
  CHECK(cuCtxGetCurrent(&ctx));
  if (ctx == NULL) return CUDA_ERROR_INVALID_CONTEXT;
  if (g_grid_mod == NULL) {
    CHECK(cuModuleLoad(&g_grid_mod, grid_cubin));
    CHECK(cuModuleGetFunction(&f_iter_grid, g_grid_mod, "_Z16iter_grid_kerneliiPiPfS0_"));
    CHECK(cuModuleGetFunction(&f_copy_grid, g_grid_mod, "_Z20copy_img_grid_kerneliiPfPh"));
    CHECK(cuModuleGetFunction(&f_err_grid, g_grid_mod, "_Z17error_grid_kerneliiPiPfS0_S0_S0_"));
  }
  if (g_equ_mod == NULL) {
    CHECK(cuModuleLoad(&g_equ_mod, equ_cubin));
    CHECK(cuModuleGetFunction(&f_iter_equ, g_equ_mod, "_Z15iter_equ_kerneliiPiPfS0_"));
    CHECK(cuModuleGetFunction(&f_copy_equ, g_equ_mod, "_Z17copy_X_equ_kerneliiPfPh"));
    CHECK(cuModuleGetFunction(&f_err_equ, g_equ_mod, "_Z16error_equ_kerneliiPiPfS0_S0_"));
    CHECK(cuModuleGetFunction(&f_errsum_equ, g_equ_mod, "_Z20error_sum_equ_kerneliiPfS_"));
  }
  return CUDA_SUCCESS;
}

static unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

/* `iters` sweeps of the reference's in-place grid kernel. */
int refcuda_grid_sweeps(int n, int m, CUdeviceptr mask, CUdeviceptr tgt, CUdeviceptr grad,
                        int grid_x, int grid_y, int iters, CUstream stream) {
  if (f_iter_grid == NULL) return CUDA_ERROR_NOT_INITIALIZED;
  void* args[] = {&n, &m, &mask, &tgt, &grad};
  const unsigned gx = ceil_div(n, grid_x), gy = ceil_div(m, grid_y);
  for (int i = 0; i < iters; ++i)
    CHECK(cuLaunchKernel(f_iter_grid, gx, gy, 1, (unsigned)grid_x, (unsigned)grid_y, 1, 0, stream,
                         args, NULL));
  return CUDA_SUCCESS;
}

/* The whole reference grid step: err cleared, sweeps, clip + residual
 * kernels, err (3 floats) and the uint8 image copied to host memory. */
int refcuda_grid_step(int n, int m, CUdeviceptr mask, CUdeviceptr tgt, CUdeviceptr grad,
                      CUdeviceptr tmp, CUdeviceptr img, CUdeviceptr err, int grid_x, int grid_y,
                      int iters, CUstream stream, float* err_host, unsigned char* img_host) {
  CHECK(cuMemsetD32Async(err, 0, 3, stream));
  CHECK(refcuda_grid_sweeps(n, m, mask, tgt, grad, grid_x, grid_y, iters, stream));
  CHECK(cuStreamSynchronize(stream));
  const unsigned gx = ceil_div(n, grid_x), gy = ceil_div(m, grid_y);
  void* cargs[] = {&n, &m, &tgt, &img};
  CHECK(cuLaunchKernel(f_copy_grid, gx, gy, 1, (unsigned)grid_x, (unsigned)grid_y, 1, 0, stream,
                       cargs, NULL));
  void* eargs[] = {&n, &m, &mask, &tgt, &grad, &tmp, &err};
  CHECK(cuLaunchKernel(f_err_grid, gx, gy, 1, (unsigned)grid_x, (unsigned)grid_y, 1, 0, stream,
                       eargs, NULL));
  CHECK(cuStreamSynchronize(stream));
  CHECK(cuMemcpyDtoH(err_host, err, 3 * sizeof(float)));
  CHECK(cuMemcpyDtoH(img_host, img, (size_t)n * m * 3));
  return CUDA_SUCCESS;
}

/* `iters` sweeps of the reference's in-place equation kernel over rows
 * 1..N-1 (row 0 is the system's unused slot). */
int refcuda_equ_sweeps(int N, CUdeviceptr A, CUdeviceptr B, CUdeviceptr X, int block_size,
                       int iters, CUstream stream) {
  if (f_iter_equ == NULL) return CUDA_ERROR_NOT_INITIALIZED;
  int n0 = 1;
  void* args[] = {&n0, &N, &A, &B, &X};
  const unsigned grid = ceil_div(N - 1, block_size);
  for (int i = 0; i < iters; ++i)
    CHECK(cuLaunchKernel(f_iter_equ, grid, 1, 1, (unsigned)block_size, 1, 1, 0, stream, args, NULL));
  return CUDA_SUCCESS;
}

int refcuda_equ_step(int N, CUdeviceptr A, CUdeviceptr B, CUdeviceptr X, CUdeviceptr tmp,
                     CUdeviceptr img, CUdeviceptr err, int block_size, int iters, CUstream stream,
                     float* err_host, unsigned char* img_host) {
  CHECK(cuMemsetD32Async(err, 0, 3, stream));
  CHECK(refcuda_equ_sweeps(N, A, B, X, block_size, iters, stream));
  CHECK(cuStreamSynchronize(stream));
  int c0 = 3, c1 = 3 * N, n0 = 1;
  void* cargs[] = {&c0, &c1, &X, &img};
  CHECK(cuLaunchKernel(f_copy_equ, ceil_div(3LL * N - 3, block_size), 1, 1, (unsigned)block_size, 1,
                       1, 0, stream, cargs, NULL));
  void* eargs[] = {&n0, &N, &A, &B, &X, &tmp};
  CHECK(cuLaunchKernel(f_err_equ, ceil_div(N - 1, block_size), 1, 1, (unsigned)block_size, 1, 1, 0,
                       stream, eargs, NULL));
  CHECK(cuStreamSynchronize(stream));
  void* sargs[] = {&N, &block_size, &tmp, &err};
  CHECK(cuLaunchKernel(f_errsum_equ, 1, 1, 1, (unsigned)block_size, 1, 1, 0, stream, sargs, NULL));
  CHECK(cuStreamSynchronize(stream));
  CHECK(cuMemcpyDtoH(err_host, err, 3 * sizeof(float)));
  CHECK(cuMemcpyDtoH(img_host, img, (size_t)N * 3));
  return CUDA_SUCCESS;
}
