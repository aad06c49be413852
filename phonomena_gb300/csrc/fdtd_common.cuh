// Shared device-side definitions of the fused elastic FDTD step.
//
// Physics: phonomena's displacement-stress staggered-grid scheme
// (simulation/base_solver.py:323-571).  The stresses T1..T6 are recomputed
// from u every step and never stored; each launch reads the state of step tt
// and writes the state of step tt+1 into separate buffers, so every output
// point is a pure function of the input state and the kernel has no in-step
// read/write hazards.
//
// Layout of every field array on the device (one array per component and
// buffer; all three components share the padded extents):
//   element (i, j, k) at  o0 + i*sx + j*sy + k,   i in [-1, nx], j in [-1, ny],
//   k in [-KOFF, pz-KOFF) with the (0,0,0) row start 32-byte aligned.
// The padding layers are zero and never written, so the 1-node halo of every
// stencil read exists without bounds checks.  Component extents inside that
// box follow the reference shapes (simulation/grid.py:88-110):
//   ux (nx-1, ny, nz)   uy (nx, ny-1, nz)   uz (nx, ny, nz-1)
// Material ids use the same (i, j, k) addressing with their own pitch.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace phono {

constexpr int TK = 32;  // tile width along z (the contiguous axis): one warp

struct Geo {
  int nx, ny, nz;          // mesh nodes per axis
  long long sx, sy, o0;    // field strides (elements) and offset of (0,0,0)
  long long msx, msy, mo0; // material-id strides and offset
};

// Per-axis spacing data.  F64: raw spacings (the reference divides).
// F32K: reciprocals (1/d rounded to float).  *0 are the first elements,
// which the reference's z=0 rows broadcast as scalars
// (simulation/base_solver.py:408-433,495-516).
template <class R>
struct Spacing {
  const R *fdx, *fdy, *fdz, *sdx, *sdy, *sdz;
  R fdx0, fdy0, fdz0, sdx0, sdy0, sdz0;
};

// Face-point enumeration: for component c and plane p (0 z=N, 1 y=N, 2 y=0,
// 3 x=N), faces_off[c*4+p] is the first flattened index; faces_off[12] is the
// total.  Planes are disjoint (a point on several faces belongs to the first
// plane in that order).
struct FaceTable {
  int off[13];
};

template <class R>
struct StepArgs {
  Geo g;
  Spacing<R> sp;
  const uint8_t* __restrict__ mat;
  const R* __restrict__ tab;   // 16 entries per material id
  const double* __restrict__ src;  // source sample per global step
  int nsrc;
  R* u[3][3];    // F64: [rotation][component]; F32K: [buffer][component] (2 used)
  R* v[2][3];    // F32K velocity; unused by F64
  R* c[2][3];    // F32K Kahan compensation; unused by F64
  R abc[8];      // clx[-1] ctx[-1] cty[0] cly[0] cty[-1] cly[-1] ctz[-1] clz[-1]
  R* surf;       // surface records: [slot][nx][ny]
  int record_every;
  int rec_base;  // record slot of the first record kept in surf
  int nrec_cap;
  const int* __restrict__ step_base;  // device counter: global step of step_off 0
  int step_off;
  int surface_mode, bc, source_mode;
  // tile decomposition of the box [0,nx-1) x [0,ny-1) x [0,nz-1)
  int ntj, ntk, nseg, xseg;
  int n_tile_blocks;
  FaceTable faces;
  int* __restrict__ err;  // device error flags (non-finite output etc.)
};

// arguments of the energy reduction (energy.cu)
struct EnergyArgs {
  Geo g;
  const void *ux, *uy, *uz;
  const void *vx, *vy, *vz;  // F32K: velocity arrays; F64: u_old arrays
  int f32;                   // element type of the arrays above
  double inv_dt;             // F64: 1/dt to form (u - u_old)/dt
  const double *fdx, *fdy, *fdz, *sdx, *sdy, *sdz;
  const uint8_t* mat;
  const double* tab;  // 13 doubles per material (C..., rho)
};

}  // namespace phono
