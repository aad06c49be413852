// Energy reduction of an FDTD state (FP64 accumulation, deterministic order).
//
// E_kin = 1/2 sum rho v^2 over the displacement points the interior update
// writes, E_str = 1/2 sum T . e over the stress points the reference computes
// (normal stresses at nodes, shears at edges; simulation/base_solver.py:323-433)
// with unit weights.  v is the half-step velocity: (u - u_old)/dt for the
// leapfrog state, the stored v for the velocity form.  Used only to measure the
// error of the FP32 path against the FP64 path; the reference has no energy.
//
// Pass 1 writes one partial pair per block into a scratch array; pass 2 sums
// the partials in block order in one block, so the result does not depend on
// scheduling.
#include <cstdio>

#include "fdtd_common.cuh"

namespace phono {

__device__ __forceinline__ double ld(const void* p, int f32, long long off) {
  return f32 ? (double)__ldg((const float*)p + off) : __ldg((const double*)p + off);
}

constexpr int EN_THREADS = 256;
constexpr int EN_WARPS = EN_THREADS / 32;

// One warp per (i, j) row of the mesh, lanes along k (coalesced loads of every
// array), rows dealt to the warps of the grid in a fixed order.  Spacings come
// as FP64 reciprocals (the strain is a difference times 1/spacing) and the
// material table is staged in shared memory, so a node costs FP64 multiplies
// and adds only.  Element type T of the displacement / velocity arrays.
template <class T>
__global__ void __launch_bounds__(EN_THREADS) energy_partial_kernel(EnergyArgs a, double2* __restrict__ partial) {
  extern __shared__ double etab[];  // nmat rows of 13
  for (int q = threadIdx.x; q < a.nmat * 13; q += EN_THREADS) etab[q] = __ldg(a.tab + q);
  __syncthreads();
  const Geo& g = a.g;
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const int lane = threadIdx.x & 31;
  const int nwarps = gridDim.x * EN_WARPS;
  const T* ux = (const T*)a.ux;
  const T* uy = (const T*)a.uy;
  const T* uz = (const T*)a.uz;
  const T* vx = (const T*)a.vx;
  const T* vy = (const T*)a.vy;
  const T* vz = (const T*)a.vz;
  const uint8_t* mat = a.mat;
  double ek = 0.0, es = 0.0;  // sums of rho v^2 and of T . e (the 1/2 is applied once)
  for (int r = blockIdx.x * EN_WARPS + (threadIdx.x >> 5); r < nx * ny; r += nwarps) {
    const int i = r / ny, j = r - (r / ny) * ny;
    const long long o = g.o0 + (long long)i * g.sx + (long long)j * g.sy;      // field (i, j, 0)
    const long long mo = g.mo0 + (long long)i * g.msx + (long long)j * g.msy;  // material (i, j, 0)
    // row predicates of the point sets below
    const bool ix_in = i <= nx - 3, iyz_in = i >= 1 && i <= nx - 2, ish = i <= nx - 2;
    const bool jx_in = j >= 1 && j <= ny - 2, jy_in = j >= 1 && j <= ny - 3, jsh = j <= ny - 2;
    const double rsdx = iyz_in ? __ldg(a.rsdx + i - 1) : 0.0, rfdx = ish ? __ldg(a.rfdx + i) : 0.0;
    const double rsdy = jx_in ? __ldg(a.rsdy + j - 1) : 0.0, rfdy = jsh ? __ldg(a.rfdy + j) : 0.0;
    for (int k = lane; k < nz; k += 32) {
      const long long p = o + k;
      const bool kin = k <= nz - 2, kn = k >= 1 && k <= nz - 2;
      const double rsdz = kn ? __ldg(a.rsdz + k - 1) : 0.0, rfdz = kn ? __ldg(a.rfdz + k) : 0.0;
      // kinetic energy at the interior displacement points, absorbing faces excluded
      auto vel = [&](const T* u, const T* v) {
        const double x = (double)__ldg(v + p);
        return a.vgiven ? x : ((double)__ldg(u + p) - x) * a.inv_dt;
      };
      if (ix_in && jx_in && kin) {
        const double v = vel(ux, vx);
        ek += etab[13 * mat[mo + g.msx + k] + 12] * v * v;
      }
      if (iyz_in && jy_in && kin) {
        const double v = vel(uy, vy);
        ek += etab[13 * mat[mo + g.msy + k] + 12] * v * v;
      }
      if (iyz_in && jx_in && k <= nz - 3) {
        const double v = vel(uz, vz);
        ek += etab[13 * mat[mo + k + 1] + 12] * v * v;
      }
      if (!kn) continue;  // every strain term below needs 1 <= k <= nz-2
      // strain energy: normal stresses at interior nodes
      if (iyz_in && jx_in) {
        const double* c = etab + 13 * mat[mo + k];
        const double e1 = ((double)__ldg(ux + p) - (double)__ldg(ux + p - g.sx)) * rsdx;
        const double e2 = ((double)__ldg(uy + p) - (double)__ldg(uy + p - g.sy)) * rsdy;
        const double e3 = ((double)__ldg(uz + p) - (double)__ldg(uz + p - 1)) * rsdz;
        const double t1 = c[0] * e1 + c[1] * e2 + c[2] * e3;
        const double t2 = c[3] * e1 + c[4] * e2 + c[5] * e3;
        const double t3 = c[6] * e1 + c[7] * e2 + c[8] * e3;
        es += t1 * e1 + t2 * e2 + t3 * e3;
      }
      // shears at edges
      if (iyz_in && jsh) {
        const double gam = ((double)__ldg(uy + p + 1) - (double)__ldg(uy + p)) * rfdz +
                           ((double)__ldg(uz + p + g.sy) - (double)__ldg(uz + p)) * rfdy;
        es += etab[13 * mat[mo + g.msy + k + 1] + 9] * gam * gam;
      }
      if (ish && jx_in) {
        const double gam = ((double)__ldg(ux + p + 1) - (double)__ldg(ux + p)) * rfdz +
                           ((double)__ldg(uz + p + g.sx) - (double)__ldg(uz + p)) * rfdx;
        es += etab[13 * mat[mo + g.msx + k + 1] + 10] * gam * gam;
      }
      if (ish && jsh) {
        const double gam = ((double)__ldg(ux + p + g.sy) - (double)__ldg(ux + p)) * rfdy +
                           ((double)__ldg(uy + p + g.sx) - (double)__ldg(uy + p)) * rfdx;
        es += etab[13 * mat[mo + g.msx + g.msy + k] + 11] * gam * gam;
      }
    }
  }
  __shared__ double sk[EN_THREADS], ss[EN_THREADS];
  sk[threadIdx.x] = 0.5 * ek;
  ss[threadIdx.x] = 0.5 * es;
  __syncthreads();
  for (int w = EN_THREADS / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sk[threadIdx.x] += sk[threadIdx.x + w];
      ss[threadIdx.x] += ss[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = make_double2(sk[0], ss[0]);
}

__global__ void __launch_bounds__(EN_THREADS) energy_final_kernel(const double2* __restrict__ partial, int n,
                                                                    double* __restrict__ out) {
  __shared__ double sk[EN_THREADS], ss[EN_THREADS];
  double ek = 0.0, es = 0.0;
  for (int q = threadIdx.x; q < n; q += EN_THREADS) {
    ek += partial[q].x;
    es += partial[q].y;
  }
  sk[threadIdx.x] = ek;
  ss[threadIdx.x] = es;
  __syncthreads();
  for (int w = EN_THREADS / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sk[threadIdx.x] += sk[threadIdx.x + w];
      ss[threadIdx.x] += ss[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sk[0];
    out[1] = ss[0];
  }
}

// partial must hold nblocks double2 values; out two doubles (device)
cudaError_t launch_energy(const EnergyArgs& a, double2* partial, int nblocks, double* out, cudaStream_t st) {
  const size_t smem = (size_t)a.nmat * 13 * sizeof(double);
  if (a.f32)
    energy_partial_kernel<float><<<nblocks, EN_THREADS, smem, st>>>(a, partial);
  else
    energy_partial_kernel<double><<<nblocks, EN_THREADS, smem, st>>>(a, partial);
  energy_final_kernel<<<1, EN_THREADS, 0, st>>>(partial, nblocks, out);
  return cudaGetLastError();
}

}  // namespace phono

// ---------------------------------------------------------------------------
// Allocation-free variant (phono_energy_static in include/phono.h).
//
// Same energy as energy_partial_kernel, over caller-owned dense arrays in the
// reference shapes, one block per x plane; the per-plane partials go to the
// file-scope scratch array below instead of a buffer from cudaMalloc, and
// energy_final_kernel sums them in plane order.  Host code must not pass the
// array's name to a kernel (it is a host-side stand-in): the device address
// is looked up once per device with cudaGetSymbolAddress.
// ---------------------------------------------------------------------------
#include <atomic>

#include "../../include/phono.h"

namespace phono {

static __device__ __align__(256) double2 g_energy_scratch[PHONO_ENERGY_STATIC_MAX_NX];

__global__ void __launch_bounds__(EN_THREADS) energy_plane_kernel(phono_energy_dense a, double2* __restrict__ partial) {
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const int i = blockIdx.x;
  const int f32 = a.precision == PHONO_F32K;
  const int vgiven = a.precision != PHONO_F64;
  const double inv_dt = 1.0 / a.dt;
  const unsigned nmat = (unsigned)a.nmat;
  bool bad_id = false;  // a material id at or past the table's end: no table read, NaN result
  auto ix = [&](int ii, int jj, int kk) { return ((long long)ii * ny + jj) * nz + kk; };          // ux, mat
  auto iy = [&](int ii, int jj, int kk) { return ((long long)ii * (ny - 1) + jj) * nz + kk; };    // uy
  auto iz = [&](int ii, int jj, int kk) { return ((long long)ii * ny + jj) * (nz - 1) + kk; };    // uz
  auto C = [&](int ii, int jj, int kk, int e) {
    const unsigned id = a.mat[ix(ii, jj, kk)];
    if (id >= nmat) {
      bad_id = true;
      return 0.0;
    }
    return a.table[id * 13 + e];
  };
  auto rho = [&](int ii, int jj, int kk) { return C(ii, jj, kk, 12); };
  auto vel = [&](const void* u, const void* v, long long off) {
    double x = ld(v, f32, off);
    return vgiven ? x : (ld(u, 0, off) - x) * inv_dt;
  };
  double ek = 0.0, es = 0.0;
  for (int q = threadIdx.x; q < ny * nz; q += EN_THREADS) {
    const int j = q / nz, k = q - j * nz;
    if (i <= nx - 3 && j >= 1 && j <= ny - 2 && k <= nz - 2) {
      double v = vel(a.ux, a.vx, ix(i, j, k));
      ek += 0.5 * rho(i + 1, j, k) * v * v;
    }
    if (i >= 1 && i <= nx - 2 && j >= 1 && j <= ny - 3 && k <= nz - 2) {
      double v = vel(a.uy, a.vy, iy(i, j, k));
      ek += 0.5 * rho(i, j + 1, k) * v * v;
    }
    if (i >= 1 && i <= nx - 2 && j >= 1 && j <= ny - 2 && k <= nz - 3) {
      double v = vel(a.uz, a.vz, iz(i, j, k));
      ek += 0.5 * rho(i, j, k + 1) * v * v;
    }
    if (i >= 1 && i <= nx - 2 && j >= 1 && j <= ny - 2 && k >= 1 && k <= nz - 2) {
      double e1 = (ld(a.ux, f32, ix(i, j, k)) - ld(a.ux, f32, ix(i - 1, j, k))) / a.sdx[i - 1];
      double e2 = (ld(a.uy, f32, iy(i, j, k)) - ld(a.uy, f32, iy(i, j - 1, k))) / a.sdy[j - 1];
      double e3 = (ld(a.uz, f32, iz(i, j, k)) - ld(a.uz, f32, iz(i, j, k - 1))) / a.sdz[k - 1];
      double t1 = C(i, j, k, 0) * e1 + C(i, j, k, 1) * e2 + C(i, j, k, 2) * e3;
      double t2 = C(i, j, k, 3) * e1 + C(i, j, k, 4) * e2 + C(i, j, k, 5) * e3;
      double t3 = C(i, j, k, 6) * e1 + C(i, j, k, 7) * e2 + C(i, j, k, 8) * e3;
      es += 0.5 * (t1 * e1 + t2 * e2 + t3 * e3);
    }
    if (i >= 1 && i <= nx - 2 && j <= ny - 2 && k >= 1 && k <= nz - 2) {
      double gam = (ld(a.uy, f32, iy(i, j, k + 1)) - ld(a.uy, f32, iy(i, j, k))) / a.fdz[k] +
                   (ld(a.uz, f32, iz(i, j + 1, k)) - ld(a.uz, f32, iz(i, j, k))) / a.fdy[j];
      es += 0.5 * C(i, j + 1, k + 1, 9) * gam * gam;
    }
    if (i <= nx - 2 && j >= 1 && j <= ny - 2 && k >= 1 && k <= nz - 2) {
      double gam = (ld(a.ux, f32, ix(i, j, k + 1)) - ld(a.ux, f32, ix(i, j, k))) / a.fdz[k] +
                   (ld(a.uz, f32, iz(i + 1, j, k)) - ld(a.uz, f32, iz(i, j, k))) / a.fdx[i];
      es += 0.5 * C(i + 1, j, k + 1, 10) * gam * gam;
    }
    if (i <= nx - 2 && j <= ny - 2 && k >= 1 && k <= nz - 2) {
      double gam = (ld(a.ux, f32, ix(i, j + 1, k)) - ld(a.ux, f32, ix(i, j, k))) / a.fdy[j] +
                   (ld(a.uy, f32, iy(i + 1, j, k)) - ld(a.uy, f32, iy(i, j, k))) / a.fdx[i];
      es += 0.5 * C(i + 1, j + 1, k, 11) * gam * gam;
    }
  }
  const bool any_bad = __syncthreads_or(bad_id);
  __shared__ double sk[EN_THREADS], ss[EN_THREADS];
  sk[threadIdx.x] = ek;
  ss[threadIdx.x] = es;
  __syncthreads();
  for (int w = EN_THREADS / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sk[threadIdx.x] += sk[threadIdx.x + w];
      ss[threadIdx.x] += ss[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[i] = any_bad ? make_double2(__longlong_as_double(0x7ff8000000000000LL),
                                                            __longlong_as_double(0x7ff8000000000000LL))
                                             : make_double2(sk[0], ss[0]);
}

}  // namespace phono

namespace phono {
void set_last_error(const char* msg);  // api.cu: message behind phono_last_error()
}

namespace {
// Device address of g_energy_scratch, looked up on the first call made with
// that device current.  Two host threads making their first call on one
// device at the same time both look it up and store the same value; the
// atomics make that well defined.  The address belongs to the device's
// primary context: after cudaDeviceReset the cache is stale, so a process
// that resets a device must not call phono_energy_static on it again.
constexpr int kMaxDevices = 64;
std::atomic<void*> g_scratch_addr[kMaxDevices];
}  // namespace

extern "C" int phono_energy_static(const phono_energy_dense* in, double* out_dev, void* stream) {
  using namespace phono;
  auto fail = [](int code, const char* msg) {
    set_last_error(msg);
    return code;
  };
  if (!in || !out_dev) return fail(PHONO_ERR_ARG, "NULL argument");
  if (in->nx < 3 || in->ny < 3 || in->nz < 3) return fail(PHONO_ERR_ARG, "nx, ny, nz must be >= 3 mesh nodes");
  if (in->nx > PHONO_ENERGY_STATIC_MAX_NX)
    return fail(PHONO_ERR_ARG, "nx exceeds PHONO_ENERGY_STATIC_MAX_NX, the planes of the static scratch array");
  if ((long long)in->ny * in->nz > 0x7fffffffLL) return fail(PHONO_ERR_ARG, "ny * nz too large");
  if (in->precision != PHONO_F64 && in->precision != PHONO_F32K && in->precision != PHONO_F64V)
    return fail(PHONO_ERR_ARG, "unknown precision");
  if (!in->ux || !in->uy || !in->uz || !in->vx || !in->vy || !in->vz || !in->mat || !in->table || !in->fdx ||
      !in->fdy || !in->fdz || !in->sdx || !in->sdy || !in->sdz)
    return fail(PHONO_ERR_ARG, "NULL device pointer in the input");
  if (!(in->dt > 0.0)) return fail(PHONO_ERR_ARG, "dt must be > 0");
  if (in->nmat < 1 || in->nmat > 256) return fail(PHONO_ERR_ARG, "nmat must be in 1..256");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(PHONO_ERR_CUDA, "cudaGetDevice failed");
  void* addr = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!addr) {
    cudaError_t e = cudaGetSymbolAddress(&addr, g_energy_scratch);
    if (e != cudaSuccess || !addr) return fail(PHONO_ERR_CUDA, "cudaGetSymbolAddress of the energy scratch failed");
    g_scratch_addr[dev].store(addr, std::memory_order_release);
  }
  double2* partial = static_cast<double2*>(addr);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  energy_plane_kernel<<<in->nx, EN_THREADS, 0, st>>>(*in, partial);
  energy_final_kernel<<<1, EN_THREADS, 0, st>>>(partial, in->nx, out_dev);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(PHONO_ERR_CUDA, cudaGetErrorString(e));
  return PHONO_OK;
}
