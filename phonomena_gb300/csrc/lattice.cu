// Material ids of a seeded phononic crystal built on the device
// (phono_set_lattice in include/phono.h): a square lattice of vertical
// cylindrical holes from the surface z = 0 down through `depth` nodes, one
// radius and one material id per lattice cell.  Replaces building the per-node
// id array on the host (the reference fills its per-node constants in a Python
// loop over inclusion nodes, simulation/material.py:59-63 with
// simulation/grid.py:158-175).  The inside test is the host builder's, in the
// same FP64 operations, so both give the same ids.
#include <cstdint>
#include "fdtd_common.cuh"

namespace phono {

// one thread per (i, j) column of nodes
__global__ void lattice_ids_kernel(uint8_t* __restrict__ mat, const Geo g, int pitch, int ncx, int ncy,
                                   const double* __restrict__ radius, const uint8_t* __restrict__ kind, int kmax,
                                   uint8_t host) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= g.ny || i >= g.nx) return;
  const int px = min(i / pitch, ncx - 1), py = min(j / pitch, ncy - 1);
  const double cx = __dmul_rn((double)px + 0.5, (double)pitch), cy = __dmul_rn((double)py + 0.5, (double)pitch);
  const double dx = __dsub_rn((double)i, cx), dy = __dsub_rn((double)j, cy);
  const double r = radius[px * ncy + py];
  const bool inside = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)) < __dmul_rn(r, r);
  const uint8_t id = inside ? kind[px * ncy + py] : host;
  uint8_t* col = mat + g.mo0 + (long long)i * g.msx + (long long)j * g.msy;
  for (int k = 0; k < g.nz; k++) col[k] = k <= kmax ? id : host;
}

cudaError_t launch_lattice_ids(uint8_t* mat, const Geo& g, int pitch, int ncx, int ncy, const double* radius,
                               const uint8_t* kind, int depth, uint8_t host, cudaStream_t st) {
  const int kmax = depth < g.nz - 1 ? depth : g.nz - 1;
  dim3 grid((g.ny + 127) / 128, g.nx);
  lattice_ids_kernel<<<grid, 128, 0, st>>>(mat, g, pitch, ncx, ncy, radius, kind, kmax, host);
  return cudaGetLastError();
}

// Material ids of the reference's inclusion model (phono_set_inclusions in
// include/phono.h): vertical cylinders (x, y, r) in mesh coordinates, each
// over a prefix [0, kend) of the z nodes.  A column (i, j) is inside
// inclusion t when sqrt((x_i - tx)^2 + (y_j - ty)^2) < r, in the FP64
// operations NumPy performs for simulation/grid.py:163-169 (the float32
// target fields widened to double, correctly rounded sqrt).  Where
// inclusions overlap, the later one in the list wins, as the reference's fill
// loop overwrites in list order (simulation/material.py:59-63).  One thread
// per column walks the list backwards and hands each newly covered stretch
// of z nodes to the inclusion that covers it; the rest of the column is
// `host`.
__global__ void inclusion_ids_kernel(uint8_t* __restrict__ mat, const Geo g, const double* __restrict__ x,
                                     const double* __restrict__ y, const double4* __restrict__ incl,
                                     const int* __restrict__ kend, const uint8_t* __restrict__ id, int n,
                                     uint8_t host) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= g.ny || i >= g.nx) return;
  const double xi = x[i], yj = y[j];
  uint8_t* col = mat + g.mo0 + (long long)i * g.msx + (long long)j * g.msy;
  int cur = 0;  // z nodes [0, cur) already assigned
  for (int t = n - 1; t >= 0 && cur < g.nz; t--) {
    const int ke = min(kend[t], g.nz);
    if (ke <= cur) continue;
    const double4 c = incl[t];  // tx, ty, r, -
    const double dx = __dsub_rn(xi, c.x), dy = __dsub_rn(yj, c.y);
    const double R = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    if (!(R < c.z)) continue;
    const uint8_t v = id[t];
    for (int k = cur; k < ke; k++) col[k] = v;
    cur = ke;
  }
  for (int k = cur; k < g.nz; k++) col[k] = host;
}

cudaError_t launch_inclusion_ids(uint8_t* mat, const Geo& g, const double* x, const double* y, const double4* incl,
                                 const int* kend, const uint8_t* id, int n, uint8_t host, cudaStream_t st) {
  dim3 grid((g.ny + 127) / 128, g.nx);
  inclusion_ids_kernel<<<grid, 128, 0, st>>>(mat, g, x, y, incl, kend, id, n, host);
  return cudaGetLastError();
}

}  // namespace phono
