/*
 * ORACLE (test infrastructure only): C restatement of fpie's strict-Jacobi
 * solvers, multi-threaded with OpenMP.  Only tests, the smoke check and the
 * CPU-baseline legs of bench.py load it; the backend never does.
 *
 * Follows the numpy backend's arithmetic order exactly, so float32 states are
 * bit-identical to the reference's numpy solvers:
 *   grid sweep     fpie/np_solver.py:81-88   x' = (g + up + down + left + right) / 4
 *   grid residual  fpie/np_solver.py:90-96   r  = 4x - g - up - down - left - right
 *   equ sweep      fpie/np_solver.py:33-41   X' = (B + X[A0] + X[A1] + X[A2] + X[A3]) / 4
 *   equ residual   fpie/np_solver.py:42-50   r  = B + X[A0] + X[A1] + X[A2] + X[A3] - 4X
 *   clip           fpie/np_solver.py:51-54, 98-101 plus the uint8 store of
 *                  fpie/process.py:278, 393 (clamp to [0,255], truncate)
 * Threading follows the reference OpenMP grid solver's static row split
 * (fpie/core/openmp/grid.cc:75-103), with rows as the unit of work.
 * Per-channel errors are accumulated in double.
 *
 * Layout is the reference's interleaved one: x[(i*m + j)*3 + c].
 * A neighbour outside the grid contributes nothing (numpy semantics).
 * Build: gcc -O3 -fopenmp -ffp-contract=off -fPIC -shared.
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <string.h>

static inline float nb(const float* x, int n, int m, int i, int j, int c) {
  if (i < 0 || i >= n || j < 0 || j >= m) return 0.0f;
  return x[((int64_t)i * m + j) * 3 + c];
}

/* iters Jacobi sweeps; x holds the state, tmp is scratch of the same size.
 * Returns 0 if the final state is in x, 1 if it is in tmp (caller copies). */
int oracle_grid_sweeps(int n, int m, const int32_t* mask, float* x, float* tmp,
                       const float* grad, int iters, int threads) {
  if (threads > 0) omp_set_num_threads(threads);
  memcpy(tmp, x, sizeof(float) * (size_t)n * m * 3);
  float* cur = x;
  float* nxt = tmp;
  for (int it = 0; it < iters; ++it) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      for (int j = 0; j < m; ++j) {
        int64_t p = (int64_t)i * m + j;
        if (!mask[p]) continue;
        for (int c = 0; c < 3; ++c) {
          float s = grad[p * 3 + c] + nb(cur, n, m, i - 1, j, c);
          s = s + nb(cur, n, m, i + 1, j, c);
          s = s + nb(cur, n, m, i, j - 1, c);
          s = s + nb(cur, n, m, i, j + 1, c);
          nxt[p * 3 + c] = s / 4.0f;
        }
      }
    }
    float* t = cur;
    cur = nxt;
    nxt = t;
  }
  return cur == x ? 0 : 1;
}

void oracle_grid_residual(int n, int m, const int32_t* mask, const float* x,
                          const float* grad, double* err, float* absr) {
  double e0 = 0, e1 = 0, e2 = 0;
#pragma omp parallel for schedule(static) reduction(+ : e0, e1, e2)
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < m; ++j) {
      int64_t p = (int64_t)i * m + j;
      float a[3] = {0, 0, 0};
      if (mask[p]) {
        for (int c = 0; c < 3; ++c) {
          float r = 4.0f * x[p * 3 + c] - grad[p * 3 + c];
          r = r - nb(x, n, m, i - 1, j, c);
          r = r - nb(x, n, m, i + 1, j, c);
          r = r - nb(x, n, m, i, j - 1, c);
          r = r - nb(x, n, m, i, j + 1, c);
          a[c] = fabsf(r);
        }
      }
      if (absr) {
        absr[p * 3 + 0] = a[0];
        absr[p * 3 + 1] = a[1];
        absr[p * 3 + 2] = a[2];
      }
      e0 += a[0];
      e1 += a[1];
      e2 += a[2];
    }
  }
  err[0] = e0;
  err[1] = e1;
  err[2] = e2;
}

void oracle_clip_u8(int64_t count, const float* x, uint8_t* out) {
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < count; ++k) {
    float v = x[k];
    out[k] = (uint8_t)(v < 0.0f ? 0.0f : (v > 255.0f ? 255.0f : v));
  }
}

int oracle_equ_sweeps(int N, const int32_t* A, float* X, float* tmp,
                      const float* B, int iters, int threads) {
  if (threads > 0) omp_set_num_threads(threads);
  float* cur = X;
  float* nxt = tmp;
  for (int it = 0; it < iters; ++it) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
      const int32_t* a = A + (int64_t)i * 4;
      for (int c = 0; c < 3; ++c) {
        float s = B[(int64_t)i * 3 + c] + cur[(int64_t)a[0] * 3 + c];
        s = s + cur[(int64_t)a[1] * 3 + c];
        s = s + cur[(int64_t)a[2] * 3 + c];
        s = s + cur[(int64_t)a[3] * 3 + c];
        nxt[(int64_t)i * 3 + c] = s / 4.0f;
      }
    }
    float* t = cur;
    cur = nxt;
    nxt = t;
  }
  return cur == X ? 0 : 1;
}

/* Red-black Gauss-Seidel of the reference's OpenMP EquSolver
 * (fpie/core/openmp/equ.cc:67-80, 107-118): rows 1..n_mid-1, then rows
 * n_mid..N-1, each updated in place; X is N x 3 interleaved. */
void oracle_equ_rb_sweeps(int N, int n_mid, const int32_t* A, float* X, const float* B, int iters,
                          int threads) {
  if (threads > 0) omp_set_num_threads(threads);
  for (int it = 0; it < iters; ++it) {
    for (int half = 0; half < 2; ++half) {
      const int lo = half ? n_mid : 1, hi = half ? N : n_mid;
#pragma omp parallel for schedule(static)
      for (int i = lo; i < hi; ++i) {
        const int32_t* a = A + (int64_t)i * 4;
        for (int c = 0; c < 3; ++c) {
          float s = B[(int64_t)i * 3 + c] + X[(int64_t)a[0] * 3 + c];
          s = s + X[(int64_t)a[1] * 3 + c];
          s = s + X[(int64_t)a[2] * 3 + c];
          s = s + X[(int64_t)a[3] * 3 + c];
          X[(int64_t)i * 3 + c] = s / 4.0f;
        }
      }
    }
  }
}

void oracle_equ_residual(int N, const int32_t* A, const float* X,
                         const float* B, double* err) {
  double e0 = 0, e1 = 0, e2 = 0;
#pragma omp parallel for schedule(static) reduction(+ : e0, e1, e2)
  for (int i = 0; i < N; ++i) {
    const int32_t* a = A + (int64_t)i * 4;
    float r[3];
    for (int c = 0; c < 3; ++c) {
      float s = B[(int64_t)i * 3 + c] + X[(int64_t)a[0] * 3 + c];
      s = s + X[(int64_t)a[1] * 3 + c];
      s = s + X[(int64_t)a[2] * 3 + c];
      s = s + X[(int64_t)a[3] * 3 + c];
      r[c] = fabsf(s - 4.0f * X[(int64_t)i * 3 + c]);
    }
    e0 += r[0];
    e1 += r[1];
    e2 += r[2];
  }
  err[0] = e0;
  err[1] = e1;
  err[2] = e2;
}
