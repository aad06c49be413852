// Shared definitions of the fused elastic FDTD step (device and host side).
//
// Physics: phonomena's displacement-stress staggered-grid scheme
// (simulation/base_solver.py:323-571).  The stresses T1..T6 are recomputed
// from u every step and never stored; each launch reads the state of step tt
// and writes the state of step tt+1 into separate buffers, so every output
// point is a pure function of the input state and the kernel has no in-step
// read/write hazards.
//
// Layout of the displacement fields on the device: one allocation holding
// nbuf x 3 arrays (buffer-major, then component ux, uy, uz), each with the
// padded extents
//   element (i, j, k) at  o0 + i*sx + j*sy + k,   i in [-1, nx], j in [-1, ny],
//   k in [-KOFF, sy-KOFF) with the (0,0,0) row start 32-byte aligned,
// so that one 4-D TMA box (k, j, i, component) loads a plane tile of all three
// components.  The padding is zero and never written: the 1-node halo of every
// stencil read exists without bounds checks.  Component extents inside that
// box follow the reference shapes (simulation/grid.py:88-110):
//   ux (nx-1, ny, nz)   uy (nx, ny-1, nz)   uz (nx, ny, nz-1)
// Material ids (uint8) use the same (i, j, k) addressing with their own
// pitch and an 8-byte front pad in k.
#pragma once
#include <cuda.h>
#include <cstdint>
#include <cuda_runtime.h>

#include "div_table.cuh"

namespace phono {

constexpr int TK = 32;      // tile width along z (the contiguous axis): one warp
constexpr int NSLOT = 4;    // planes in the shared-memory ring
constexpr int SEG_TABLE = 64;  // x segments a launch describes by table (more: uniform segments)
constexpr int MKOFF = 8;    // material front pad in k (bytes)
constexpr int MKW = 48;     // material tile width in k (bytes): k0-8 .. k0+40
constexpr int TAB_ROWS_MAX = 256;  // material rows a table may hold (uint8 ids)
constexpr int BATCH_TAB_ROWS = 32;  // material rows of a batched instance

template <class R>
struct Lay;
template <>
struct Lay<double> {
  static constexpr int KOFF = 4;   // field front pad in k (elements): 32 bytes
  static constexpr int KW = 36;    // tile width in k: k0-2 .. k0+34 (288 bytes)
  static constexpr int KB = 2;     // column of k0 inside the tile
};
template <>
struct Lay<float> {
  static constexpr int KOFF = 8;
  static constexpr int KW = 40;    // k0-4 .. k0+36 (160 bytes)
  static constexpr int KB = 4;
};

struct Geo {
  int nx, ny, nz;          // mesh nodes per axis
  long long sx, sy, o0;    // field strides (elements) and offset of (0,0,0)
  long long fstride;       // elements between consecutive field arrays
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
// 3 x=N), off[c*4+p] is the first flattened index; off[12] is the total.
// Planes are disjoint (a point on several faces belongs to the first plane in
// that order).  Plane 0 lists only the z=N points that also lie on an x or y
// face: the tile pass writes the others.
struct FaceTable {
  int off[13];
};

template <class R>
struct StepArgs {
  CUtensorMap tm_u;    // 4-D (k, j, i, buffer*3+component) map of the u allocation
  CUtensorMap tm_mat;  // 3-D (k, j, i) map of the material ids
  CUtensorMap tm_pw0;  // own-point tiles of u_old (F64) or v (velocity forms), same layout as tm_u
  CUtensorMap tm_pw1;  // own-point tiles of the Kahan terms (velocity forms)
  Geo g;
  Spacing<R> sp;
  DivTable dtab;
  const uint8_t* __restrict__ mat;
  const R* __restrict__ tab;       // 16 entries per material id
  int nmat;
  const double* __restrict__ src;  // source sample per global step
  R* ubase;      // u allocation: array (buffer*3 + c) at ubase + (buffer*3+c)*fstride
  R* vbase;      // F32K velocity arrays (2 buffers x 3), same layout
  R* cbase;      // F32K Kahan compensation arrays
  R abc[8];      // clx[-1] ctx[-1] cty[0] cly[0] cty[-1] cly[-1] ctz[-1] clz[-1]
  R dt;          // time step (the table's column 14, the same for every material)
  R* surf;       // surface records: [slot][nx][ny]
  int record_every;
  int rec_base;  // record slot of the first record kept in surf
  int nrec_cap;
  const int* __restrict__ step_base;  // device counter: global step of step_off 0
  int step_off;
  int surface_mode, bc, source_mode;
  // tile decomposition of the box [0,nx-1) x [0,ny-1) x [0,nz-1)
  int ntj, ntk, nseg, xseg;
  // first plane of each x segment (nseg + 1 entries) when nseg <= SEG_TABLE;
  // the segment order is the launch order, so short segments can come last
  int seg_start[SEG_TABLE + 1];
  int n_tile_blocks;
  FaceTable faces;
  int* __restrict__ err;  // device error flags: 1 non-finite surface value, 2 pipeline wait timed out
  int step_end;           // global steps >= step_end are skipped (a batched instance's budget)
  // Bounded waits of the tile pass: polls of an mbarrier before the wait
  // gives up (0: the default budget, about 0.3 s).  skip_plane >= 0 is a test
  // hook: blocks arm that plane's barrier but issue no copy for it, so the
  // wait on it runs out and the time-out path (error bit 2, drain, return)
  // runs.  -1 in production.
  int wait_polls;
  int skip_plane;
};

// Batched launch: many instances (each a StepArgs in device memory) share one
// persistent tile launch and one face launch per step.
template <class R>
struct BatchArgs {
  const StepArgs<R>* inst;  // [capacity] per-instance arguments
  const int2* items;        // (instance, tile) work items, costliest first
  const int* counts;        // [0] work items, [1] face blocks, [2] entries of face_prefix
  unsigned* ticket;         // work-item counter; returns to 0 after every launch
  const int* face_prefix;   // first face block of each listed instance (+ total)
  const int* face_inst;     // instance of each listed entry
  const int* active;        // [counts[3]] active instances (step-counter update)
  int step_off;             // offset of this launch inside a captured chunk of steps
};

// arguments of the energy reduction (energy.cu)
struct EnergyArgs {
  Geo g;
  const void *ux, *uy, *uz;
  const void *vx, *vy, *vz;  // F32K: velocity arrays; F64: u_old arrays
  int f32;                   // element type of the arrays above (float / double)
  int vgiven;                // vx.. hold the velocity (velocity forms) rather than u_old
  double inv_dt;             // F64: 1/dt to form (u - u_old)/dt
  const double *rfdx, *rfdy, *rfdz, *rsdx, *rsdy, *rsdz;  // reciprocal spacings 1/fd, 1/sd
  const uint8_t* mat;
  const double* tab;  // 13 doubles per material (C..., rho)
  int nmat;           // rows of tab
};

}  // namespace phono
