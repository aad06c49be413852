// GPU check of the FP64 leapfrog's division: div_tab (the device code the
// step kernels use, phonomena_gb300/csrc/div_table.cuh) against __ddiv_rn,
// bit for bit, on operand pairs the test chooses.  Test infrastructure only:
// built into its own small library by phonomena_gb300/build.py and loaded by
// tests/test_gpu_division.py.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "div_table.cuh"

namespace {

__global__ void div_check_kernel(const double* __restrict__ x, const double* __restrict__ b, long long n,
                                 phono::DivTable t, unsigned long long* bad, double* first_bad_x) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const double want = __ddiv_rn(x[q], b[q]);
    const double got = phono::div_tab(x[q], b[q], t);
    const bool same = __double_as_longlong(want) == __double_as_longlong(got) || (isnan(want) && isnan(got));
    if (!same && atomicAdd(bad, 1ull) == 0ull) *first_bad_x = x[q];
  }
}

}  // namespace

// Divide x[i] by b[i] (n pairs) through a divisor table built over the
// distinct b (as phono_create builds it for a mesh) and count the quotients
// that differ from IEEE division.  out: [0] mismatches, [1] table entries,
// [2] entries marked exact (two-operation quotient), [3] the first
// mismatching x (as bits).  Returns 0, or -1 when no table could be built,
// -2 on a CUDA error.
extern "C" int div_check_gpu(const double* x, const double* b, long long n, unsigned long long out[4]) {
  std::vector<double> tbl;
  phono::DivTable t{};
  if (!phono::build_div_table(std::vector<double>(b, b + n), tbl, &t.mult, &t.shift)) return -1;
  unsigned long long entries = 0, exact = 0;
  for (size_t s = 0; s < tbl.size(); s += 4) {
    uint64_t u;
    std::memcpy(&u, &tbl[s], 8);
    if (u != ~0ull) {
      entries++;
      exact += tbl[s + 3] != 0.0;
    }
  }
  double *dx = nullptr, *db = nullptr, *dt = nullptr, *dfirst = nullptr;
  unsigned long long* dbad = nullptr;
  int rc = 0;
  unsigned long long bad = 0;
  double first = 0.0;
  if (cudaMalloc(&dx, n * 8) != cudaSuccess || cudaMalloc(&db, n * 8) != cudaSuccess ||
      cudaMalloc(&dt, tbl.size() * 8) != cudaSuccess || cudaMalloc(&dbad, 8) != cudaSuccess ||
      cudaMalloc(&dfirst, 8) != cudaSuccess ||
      cudaMemcpy(dx, x, n * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(db, b, n * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dt, tbl.data(), tbl.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(dbad, 0, 8) != cudaSuccess || cudaMemset(dfirst, 0, 8) != cudaSuccess) {
    rc = -2;
  } else {
    t.tab = dt;
    div_check_kernel<<<1216, 256>>>(dx, db, n, t, dbad, dfirst);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(&bad, dbad, 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&first, dfirst, 8, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = -2;
  }
  cudaFree(dx);
  cudaFree(db);
  cudaFree(dt);
  cudaFree(dbad);
  cudaFree(dfirst);
  uint64_t fb;
  std::memcpy(&fb, &first, 8);
  out[0] = bad;
  out[1] = entries;
  out[2] = exact;
  out[3] = fb;
  return rc;
}

// Host only (no CUDA call): the divisor table build_div_table makes for
// `values`, for checking the host code on a machine without a GPU.
// table_out: 4 * slots doubles ({b, yh, yl, exact} per slot, empty slots all
// ones); returns the slot count, 0 when no table was built.
extern "C" int div_table_host(const double* values, int n, double* table_out, int table_cap, unsigned* mult,
                              int* shift) {
  std::vector<double> tbl;
  if (!phono::build_div_table(std::vector<double>(values, values + n), tbl, mult, shift)) return 0;
  if ((int)tbl.size() > table_cap) return -1;
  std::memcpy(table_out, tbl.data(), tbl.size() * sizeof(double));
  return (int)(tbl.size() / 4);
}
