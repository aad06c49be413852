// Elastic FDTD step for GB300 (sm_103a).
//
// One time step of phonomena's staggered-grid solver
// (simulation/base_solver.py:245-266) is a tile launch and a face launch:
//
//  * tile blocks (tile_rows.cuh): a (TJ x 32) tile of the
//    (y, z) plane marches along x over a segment of planes.  Planes of u (all
//    three components, 1-node halo), of the material ids and of the pointwise
//    state of the own points (u_old, or v and the Kahan term) stream into a
//    4-slot shared-memory ring through TMA (cp.async.bulk.tensor, completion
//    on an mbarrier per slot).  Each iteration evaluates the six stresses of
//    the current plane once (plus the halo stresses the neighbours need) into
//    shared memory and writes the new state of the plane.  Stresses are never
//    written to global memory.  The tile pass also writes the z = N face
//    point above every (i, j) that is on no x / y face.
//
//  * face points (fdtd_face_kernel, a second launch; for ny == 3, extra
//    blocks of the same launch): the x = N, y = 0, y = N faces and the z = N
//    points on them (simulation/base_solver.py:540-554).  The reference
//    applies the faces one after another, each reading the plane next to it
//    as left by the earlier faces; the final value of a face point is thus a
//    chain of at most four face formulas ending at the interior value of one
//    point q.  The face thread walks that chain from q's new value (written
//    by the tile pass; evaluated from the input state in the one-launch form).
//
// Three arithmetic schemes share this structure:
//  F64  - the reference leapfrog u' = (2u - u_old) + (dt^2/P) * div T with the
//         reference's IEEE operation order (explicit _rn intrinsics, true
//         division), bit-identical to the reference CPU solver.
//  F32K - FP32 velocity form v' = v + (dt/P) div T, u' = u + dt v' with a
//         Kahan-compensated displacement sum; explicit fmaf only.
//  F64V - the F32K scheme in FP64.
//
// Batches (batch_step_kernel and friends) run the same tile pass over the
// (instance, tile) work items of many instances in one persistent launch.
#include <cstdio>
#include "fdtd_common.cuh"

namespace phono {

// ---------------------------------------------------------------------------
// arithmetic schemes
// ---------------------------------------------------------------------------
struct F64 {
  using R = double;
  static constexpr bool kahan = false;
  __device__ __forceinline__ static R sub(R a, R b) { return __dsub_rn(a, b); }
  // x / b with IEEE rounding, through the divisor table when the handle has one
  __device__ __forceinline__ static R dv(const DivTable& k, R x, R b) { return k.tab ? div_tab(x, b, k) : __ddiv_rn(x, b); }
  // normal stresses ((C0*d1)/a + (C1*d2)/b) + (C2*d3)/d   (base_solver.py:329-351)
  __device__ __forceinline__ static R tn1(const DivTable& k, const R* c, R d1, R d2, R d3, R a, R b, R d) {
    return __dadd_rn(__dadd_rn(dv(k, __dmul_rn(c[0], d1), a), dv(k, __dmul_rn(c[1], d2), b)),
                     dv(k, __dmul_rn(c[2], d3), d));
  }
  // shear stress C * (d1/a + d2/b)   (base_solver.py:353-372)
  __device__ __forceinline__ static R ts(const DivTable& k, R cs, R d1, R a, R d2, R b) {
    return __dmul_rn(cs, __dadd_rn(dv(k, d1, a), dv(k, d2, b)));
  }
  // (d1/a + d2/b) + d3/c   (base_solver.py:444-446)
  __device__ __forceinline__ static R div3(const DivTable& k, R d1, R a, R d2, R b, R d3, R c) {
    return __dadd_rn(__dadd_rn(dv(k, d1, a), dv(k, d2, b)), dv(k, d3, c));
  }
  // uz z=0 row as written at base_solver.py:516: ((d1/a + d2/b) + T3[..,1]) - T3[..,0]/fdz
  // with T3[..,0] == +0, so the last subtraction is exact and dropped.
  __device__ __forceinline__ static R div_surf_ref(const DivTable& k, R d1, R a, R d2, R b, R t31) {
    return __dadd_rn(__dadd_rn(dv(k, d1, a), dv(k, d2, b)), t31);
  }
  // u[b-+1] + c * (u_new[b-+1] - u[b])   (base_solver.py:540-554)
  __device__ __forceinline__ static R abc(R coef, R nbr_new, R self_old, R nbr_old) {
    return __dadd_rn(nbr_old, __dmul_rn(coef, __dsub_rn(nbr_new, self_old)));
  }
};

struct F32K {
  using R = float;
  static constexpr bool kahan = true;
  __device__ __forceinline__ static R sub(R a, R b) { return __fsub_rn(a, b); }
  // strains e = d * (1/spacing); T = fmaf(C0, e1, fmaf(C1, e2, C2 * e3))
  __device__ __forceinline__ static R tn1(const DivTable&, const R* c, R d1, R d2, R d3, R a, R b, R d) {
    return __fmaf_rn(c[0], __fmul_rn(d1, a), __fmaf_rn(c[1], __fmul_rn(d2, b), __fmul_rn(c[2], __fmul_rn(d3, d))));
  }
  __device__ __forceinline__ static R ts(const DivTable&, R cs, R d1, R a, R d2, R b) {
    return __fmul_rn(cs, __fmaf_rn(d1, a, __fmul_rn(d2, b)));
  }
  __device__ __forceinline__ static R div3(const DivTable&, R d1, R a, R d2, R b, R d3, R c) {
    return __fmaf_rn(d1, a, __fmaf_rn(d2, b, __fmul_rn(d3, c)));
  }
  // reference-precedence z = 0 row: T3[..,1] as the third term with factor 1
  __device__ __forceinline__ static R div_surf_ref(const DivTable& k, R d1, R a, R d2, R b, R t31) {
    return div3(k, d1, a, d2, b, t31, 1.0f);
  }
  __device__ __forceinline__ static R abc(R coef, R nbr_new, R self_old, R nbr_old) {
    return __fmaf_rn(coef, __fsub_rn(nbr_new, self_old), nbr_old);
  }
  __device__ __forceinline__ static R fma(R a, R b, R c) { return __fmaf_rn(a, b, c); }
  __device__ __forceinline__ static R add(R a, R b) { return __fadd_rn(a, b); }
};

// The F32K scheme carried out in FP64: the fast FP64 reference for judging
// the FP32 error (same operation sequence, double rounding).
struct F64V {
  using R = double;
  static constexpr bool kahan = true;
  __device__ __forceinline__ static R sub(R a, R b) { return __dsub_rn(a, b); }
  __device__ __forceinline__ static R tn1(const DivTable&, const R* c, R d1, R d2, R d3, R a, R b, R d) {
    return __fma_rn(c[0], __dmul_rn(d1, a), __fma_rn(c[1], __dmul_rn(d2, b), __dmul_rn(c[2], __dmul_rn(d3, d))));
  }
  __device__ __forceinline__ static R ts(const DivTable&, R cs, R d1, R a, R d2, R b) {
    return __dmul_rn(cs, __fma_rn(d1, a, __dmul_rn(d2, b)));
  }
  __device__ __forceinline__ static R div3(const DivTable&, R d1, R a, R d2, R b, R d3, R c) {
    return __fma_rn(d1, a, __fma_rn(d2, b, __dmul_rn(d3, c)));
  }
  __device__ __forceinline__ static R div_surf_ref(const DivTable& k, R d1, R a, R d2, R b, R t31) {
    return div3(k, d1, a, d2, b, t31, 1.0);
  }
  __device__ __forceinline__ static R abc(R coef, R nbr_new, R self_old, R nbr_old) {
    return __fma_rn(coef, __dsub_rn(nbr_new, self_old), nbr_old);
  }
  __device__ __forceinline__ static R fma(R a, R b, R c) { return __fma_rn(a, b, c); }
  __device__ __forceinline__ static R add(R a, R b) { return __dadd_rn(a, b); }
};

// ---------------------------------------------------------------------------
// addressing
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long fidx(const Geo& g, int i, int j, int k) {
  return g.o0 + (long long)i * g.sx + (long long)j * g.sy + k;
}

// component extents and face coordinates
__device__ __forceinline__ int ext_x(const Geo& g, int c) { return g.nx - (c == 0); }
__device__ __forceinline__ int ext_y(const Geo& g, int c) { return g.ny - (c == 1); }
__device__ __forceinline__ int ext_z(const Geo& g, int c) { return g.nz - (c == 2); }
__device__ __forceinline__ bool on_face(const Geo& g, int c, int i, int j, int k) {
  return i == ext_x(g, c) - 1 || j == 0 || j == ext_y(g, c) - 1 || k == ext_z(g, c) - 1;
}
// points the reference's interior update or z=0 row writes
// (base_solver.py:441-463,495-516)
__device__ __forceinline__ bool in_v0(const Geo& g, int c, int i, int j, int k) {
  if (c == 0) return j >= 1 && j <= g.ny - 2 && k >= 0 && k <= g.nz - 2;
  if (c == 1) return i >= 1 && i <= g.nx - 2 && k >= 0 && k <= g.nz - 2;
  return i >= 1 && i <= g.nx - 2 && j >= 1 && j <= g.ny - 2;
}

// ---------------------------------------------------------------------------
// stress at a point, given a fetcher F: x/y/z(i,j,k) -> u, row(i,j,k) -> the
// 16-entry material row.  Zero wherever the reference never writes the
// stress array.
// ---------------------------------------------------------------------------
template <class S, class F>
__device__ __forceinline__ typename S::R t1_at(const StepArgs<typename S::R>& a, const F& f, int i, int j, int k,
                                               int which) {  // which: 0 T1, 1 T2, 2 T3
  using R = typename S::R;
  const Geo& g = a.g;
  if (i < 1 || i > g.nx - 2 || j < 1 || j > g.ny - 2 || k < 0 || k > g.nz - 2) return R(0);
  if (k == 0 && which == 2) return R(0);  // T3[1:-1,1:-1,0] = 0 (base_solver.py:418)
  const R* c = f.row(i, j, k) + 3 * which;
  R d1 = S::sub(f.x(i, j, k), f.x(i - 1, j, k));
  R d2 = S::sub(f.y(i, j, k), f.y(i, j - 1, k));
  if (k == 0)  // base_solver.py:408-416: uz - 0, first-element spacings
    return S::tn1(a.dtab, c, d1, d2, f.z(i, j, 0), a.sp.sdx0, a.sp.sdy0, a.sp.sdz0);
  return S::tn1(a.dtab, c, d1, d2, S::sub(f.z(i, j, k), f.z(i, j, k - 1)), __ldg(a.sp.sdx + i - 1),
                __ldg(a.sp.sdy + j - 1), __ldg(a.sp.sdz + k - 1));
}

template <class S, class F>
__device__ __forceinline__ void t123_at(const StepArgs<typename S::R>& a, const F& f, int i, int j, int k,
                                        typename S::R& T1, typename S::R& T2, typename S::R& T3) {
  using R = typename S::R;
  const Geo& g = a.g;
  if (i < 1 || i > g.nx - 2 || j < 1 || j > g.ny - 2 || k < 0 || k > g.nz - 2) {
    T1 = T2 = T3 = R(0);
    return;
  }
  const R* c = f.row(i, j, k);
  R d1 = S::sub(f.x(i, j, k), f.x(i - 1, j, k));
  R d2 = S::sub(f.y(i, j, k), f.y(i, j - 1, k));
  if (k == 0) {
    R d3 = f.z(i, j, 0);
    T1 = S::tn1(a.dtab, c, d1, d2, d3, a.sp.sdx0, a.sp.sdy0, a.sp.sdz0);
    T2 = S::tn1(a.dtab, c + 3, d1, d2, d3, a.sp.sdx0, a.sp.sdy0, a.sp.sdz0);
    T3 = R(0);
  } else {
    R d3 = S::sub(f.z(i, j, k), f.z(i, j, k - 1));
    R sa = __ldg(a.sp.sdx + i - 1), sb = __ldg(a.sp.sdy + j - 1), sd = __ldg(a.sp.sdz + k - 1);
    T1 = S::tn1(a.dtab, c, d1, d2, d3, sa, sb, sd);
    T2 = S::tn1(a.dtab, c + 3, d1, d2, d3, sa, sb, sd);
    T3 = S::tn1(a.dtab, c + 6, d1, d2, d3, sa, sb, sd);
  }
}

template <class S, class F>
__device__ __forceinline__ typename S::R t4_at(const StepArgs<typename S::R>& a, const F& f, int i, int j, int k) {
  using R = typename S::R;
  const Geo& g = a.g;
  if (i < 1 || i > g.nx - 2 || j < 0 || j > g.ny - 2 || k < 0 || k > g.nz - 2) return R(0);
  if (k == 0)  // base_solver.py:420-423
    return S::ts(a.dtab, f.row(i, j + 1, 0)[9], S::sub(f.y(i, j, 1), f.y(i, j, 0)), a.sp.fdy0,
                 S::sub(f.z(i, j + 1, 0), f.z(i, j, 0)), a.sp.fdz0);
  return S::ts(a.dtab, f.row(i, j + 1, k + 1)[9], S::sub(f.y(i, j, k + 1), f.y(i, j, k)), __ldg(a.sp.fdz + k),
               S::sub(f.z(i, j + 1, k), f.z(i, j, k)), __ldg(a.sp.fdy + j));
}

template <class S, class F>
__device__ __forceinline__ typename S::R t5_at(const StepArgs<typename S::R>& a, const F& f, int i, int j, int k) {
  using R = typename S::R;
  const Geo& g = a.g;
  if (i < 0 || i > g.nx - 2 || j < 1 || j > g.ny - 2 || k < 0 || k > g.nz - 2) return R(0);
  if (k == 0)  // base_solver.py:425-428
    return S::ts(a.dtab, f.row(i + 1, j, 0)[10], S::sub(f.x(i, j, 1), f.x(i, j, 0)), a.sp.fdx0,
                 S::sub(f.z(i + 1, j, 0), f.z(i, j, 0)), a.sp.fdz0);
  return S::ts(a.dtab, f.row(i + 1, j, k + 1)[10], S::sub(f.x(i, j, k + 1), f.x(i, j, k)), __ldg(a.sp.fdz + k),
               S::sub(f.z(i + 1, j, k), f.z(i, j, k)), __ldg(a.sp.fdx + i));
}

template <class S, class F>
__device__ __forceinline__ typename S::R t6_at(const StepArgs<typename S::R>& a, const F& f, int i, int j, int k) {
  using R = typename S::R;
  const Geo& g = a.g;
  if (i < 0 || i > g.nx - 2 || j < 0 || j > g.ny - 2 || k < 0 || k > g.nz - 2) return R(0);
  if (k == 0)  // base_solver.py:430-433
    return S::ts(a.dtab, f.row(i + 1, j + 1, 0)[11], S::sub(f.x(i, j + 1, 0), f.x(i, j, 0)), a.sp.fdx0,
                 S::sub(f.y(i + 1, j, 0), f.y(i, j, 0)), a.sp.fdz0);
  return S::ts(a.dtab, f.row(i + 1, j + 1, k)[11], S::sub(f.x(i, j + 1, k), f.x(i, j, k)), __ldg(a.sp.fdy + j),
               S::sub(f.y(i + 1, j, k), f.y(i, j, k)), __ldg(a.sp.fdx + i));
}

// divergence terms of the three components (base_solver.py:441-463,495-516)
// and the material row whose density applies
template <class S, class F>
__device__ __forceinline__ typename S::R div_x(const StepArgs<typename S::R>& a, const F& f, int i, int j, int k,
                                               typename S::R t1p, typename S::R t1m, typename S::R t6a,
                                               typename S::R t6b, typename S::R t5a, typename S::R t5b,
                                               const typename S::R*& row) {
  if (k == 0) {
    row = f.row(i + 1, j, 0);
    return S::div3(a.dtab, S::sub(t1p, t1m), a.sp.fdx0, S::sub(t6a, t6b), a.sp.sdy0, t5a, a.sp.sdz0);
  }
  row = f.row(i + 1, j, k);
  return S::div3(a.dtab, S::sub(t1p, t1m), __ldg(a.sp.fdx + i), S::sub(t6a, t6b), __ldg(a.sp.sdy + j - 1),
                 S::sub(t5a, t5b), __ldg(a.sp.sdz + k - 1));
}
template <class S, class F>
__device__ __forceinline__ typename S::R div_y(const StepArgs<typename S::R>& a, const F& f, int i, int j, int k,
                                               typename S::R t6a, typename S::R t6b, typename S::R t2p,
                                               typename S::R t2m, typename S::R t4a, typename S::R t4b,
                                               const typename S::R*& row) {
  if (k == 0) {
    row = f.row(i, j + 1, 0);
    return S::div3(a.dtab, S::sub(t6a, t6b), a.sp.sdx0, S::sub(t2p, t2m), a.sp.fdy0, t4a, a.sp.sdz0);
  }
  row = f.row(i, j + 1, k);
  return S::div3(a.dtab, S::sub(t6a, t6b), __ldg(a.sp.sdx + i - 1), S::sub(t2p, t2m), __ldg(a.sp.fdy + j),
                 S::sub(t4a, t4b), __ldg(a.sp.sdz + k - 1));
}
template <class S, class F>
__device__ __forceinline__ typename S::R div_z(const StepArgs<typename S::R>& a, const F& f, int i, int j, int k,
                                               typename S::R t5a, typename S::R t5b, typename S::R t4a,
                                               typename S::R t4b, typename S::R t3p, typename S::R t3m,
                                               const typename S::R*& row) {
  if (k == 0) {
    row = f.row(i, j, 0);  // density at z index 0 (base_solver.py:513)
    if (a.surface_mode == 0) return S::div_surf_ref(a.dtab, S::sub(t5a, t5b), a.sp.sdx0, S::sub(t4a, t4b), a.sp.sdy0, t3p);
    return S::div3(a.dtab, S::sub(t5a, t5b), a.sp.sdx0, S::sub(t4a, t4b), a.sp.sdy0, t3p, a.sp.fdz0);
  }
  row = f.row(i, j, k + 1);
  return S::div3(a.dtab, S::sub(t5a, t5b), __ldg(a.sp.sdx + i - 1), S::sub(t4a, t4b), __ldg(a.sp.sdy + j - 1),
                 S::sub(t3p, t3m), __ldg(a.sp.fdz + k));
}

// state arrays of global step tt: buffer indices, pointers formed on use
// (no pointer arrays, which would live in local memory)
template <class R>
struct Roles {
  // component-0 array of each role (component c at + c * fs), set once per
  // launch: an access is the point's offset added to a block-uniform base
  R *u_cur, *u_old, *u_out, *v_in, *v_out, *c_in, *c_out;
  long long fs;
  int rold, rcur, rout;  // buffer indices: u at tt-1 (F64), tt, tt+1
  __device__ __forceinline__ const R* cur(int c) const { return u_cur + c * fs; }
  __device__ __forceinline__ const R* old(int c) const { return u_old + c * fs; }
  __device__ __forceinline__ R* out(int c) const { return u_out + c * fs; }
  __device__ __forceinline__ const R* vin(int c) const { return v_in + c * fs; }
  __device__ __forceinline__ const R* cin(int c) const { return c_in + c * fs; }
  __device__ __forceinline__ R* vout(int c) const { return v_out + c * fs; }
  __device__ __forceinline__ R* cout(int c) const { return c_out + c * fs; }
};

template <class S>
__device__ __forceinline__ Roles<typename S::R> roles(const StepArgs<typename S::R>& a, int tt) {
  Roles<typename S::R> r;
  r.fs = a.g.fstride;
  if (!S::kahan) {
    r.rold = tt % 3;
    r.rcur = (tt + 1) % 3;
    r.rout = (tt + 2) % 3;
  } else {
    r.rcur = tt & 1;
    r.rout = r.rcur ^ 1;
    r.rold = r.rcur;
  }
  const long long f3 = 3 * r.fs;
  r.u_cur = a.ubase + r.rcur * f3;
  r.u_old = a.ubase + r.rold * f3;
  r.u_out = a.ubase + r.rout * f3;
  r.v_in = a.vbase + r.rcur * f3;
  r.v_out = a.vbase + r.rout * f3;
  r.c_in = a.cbase + r.rcur * f3;
  r.c_out = a.cbase + r.rout * f3;
  return r;
}

// pointwise state of a V0 point that the update needs besides u itself
template <class R>
struct Pw {
  R p0, p1;  // F64: u_old, -; F32K: v, c
};

template <class S>
__device__ __forceinline__ Pw<typename S::R> load_pw(const Roles<typename S::R>& r, int c, long long off) {
  Pw<typename S::R> p;
  if constexpr (!S::kahan) {
    p.p0 = __ldg(r.old(c) + off);
    p.p1 = 0;
  } else {
    p.p0 = __ldg(r.vin(c) + off);
    p.p1 = __ldg(r.cin(c) + off);
  }
  return p;
}

// new state of one V0 point: F64 leapfrog / F32K Kahan velocity update.
// q = the table's column 12 at the point (dt^2/P or dt/P), dt = column 14.
template <class S>
__device__ __forceinline__ typename S::R update_value(typename S::R u, Pw<typename S::R> pw, typename S::R dv,
                                                      typename S::R q, typename S::R dt, typename S::R& vn,
                                                      typename S::R& cn) {
  using R = typename S::R;
  if constexpr (!S::kahan) {
    // (2u - u_old) + (dt^2/P) * div   (base_solver.py:441-443)
    vn = cn = 0;
    return __dadd_rn(__dsub_rn(__dmul_rn(2.0, u), pw.p0), __dmul_rn(q, dv));
  } else {
    R v2 = S::fma(q, dv, pw.p0);   // v + (dt/P) div
    R y = S::fma(dt, v2, -pw.p1);  // dt v - c
    R t = S::add(u, y);
    cn = S::sub(S::sub(t, u), y);
    vn = v2;
    return t;
  }
}
template <class S>
__device__ __forceinline__ typename S::R update_value(typename S::R u, Pw<typename S::R> pw, typename S::R dv,
                                                      const typename S::R* row, typename S::R& vn,
                                                      typename S::R& cn) {
  return update_value<S>(u, pw, dv, row[12], row[14], vn, cn);
}

// OFF: element offset inside one array; the tile path passes a 32-bit
// unsigned offset (one multiply-add per address), the face path 64-bit
template <class S, class OFF>
__device__ __forceinline__ void store_point(const Roles<typename S::R>& r, int c, OFF off, typename S::R un,
                                            typename S::R vn, typename S::R cn) {
  r.out(c)[off] = un;
  if constexpr (S::kahan) {
    r.vout(c)[off] = vn;
    r.cout(c)[off] = cn;
  }
}

// a point the reference does not write this step keeps its state; returns u
template <class S, class OFF>
__device__ __forceinline__ typename S::R store_stale(const Roles<typename S::R>& r, int c, OFF off) {
  const typename S::R u = __ldg(r.cur(c) + off);
  r.out(c)[off] = u;
  if constexpr (S::kahan) {
    r.vout(c)[off] = __ldg(r.vin(c) + off);
    r.cout(c)[off] = __ldg(r.cin(c) + off);
  }
  return u;
}

template <class R>
__device__ __forceinline__ void record(const StepArgs<R>& a, int tt, int i, int j, R val) {
  if (a.record_every > 0 && (tt + 1) % a.record_every == 0) {
    int slot = (tt + 1) / a.record_every - 1 - a.rec_base;
    if (slot >= 0 && slot < a.nrec_cap) a.surf[((long long)slot * a.g.nx + i) * a.g.ny + j] = val;
  }
  if (!isfinite(val)) atomicOr(a.err, 1);
}

// ---------------------------------------------------------------------------
// fetchers
// ---------------------------------------------------------------------------
template <class R>
struct GlobalFetch {
  const R* ux;
  const R* uy;
  const R* uz;
  const uint8_t* mat;
  const R* tab;
  Geo g;
  R s;
  int wall;
  __device__ __forceinline__ R x(int i, int j, int k) const { return __ldg(ux + fidx(g, i, j, k)); }
  __device__ __forceinline__ R y(int i, int j, int k) const { return __ldg(uy + fidx(g, i, j, k)); }
  __device__ __forceinline__ R z(int i, int j, int k) const {
    if (i == 0 && (wall || k == 0)) return s;  // source overwrite (base_solver.py:251)
    return __ldg(uz + fidx(g, i, j, k));
  }
  __device__ __forceinline__ const R* row(int i, int j, int k) const {
    return tab + 16 * __ldg(mat + g.mo0 + (long long)i * g.msx + (long long)j * g.msy + k);
  }
};

// Geometry of one ring slot of a (TJ x 32) tile: a u component tile is
// TJ+2 rows (1-row halo) of KW values starting KB before the tile's first z
// point; the three components follow each other (CW apart); SU and SM are the
// slot strides of u and of the material ids, rounded to 128 bytes.
template <class R, int TJ>
struct TileShape {
  static constexpr int KW = Lay<R>::KW, KB = Lay<R>::KB;
  static constexpr int CW = (TJ + 2) * KW;                       // component stride in a slot
  static constexpr int SU = ((3 * CW * (int)sizeof(R) + 127) / 128) * 128 / (int)sizeof(R);  // slot stride
  static constexpr int SM = (((TJ + 2) * MKW + 127) / 128) * 128;                               // mat slot stride
};

// interior (V0) value of u_new at a point, evaluated from global memory
template <class S>
__device__ typename S::R v0_global(const StepArgs<typename S::R>& a, const Roles<typename S::R>& r,
                                   const GlobalFetch<typename S::R>& f, int c, int i, int j, int k) {
  using R = typename S::R;
  const Geo& g = a.g;
  long long off = fidx(g, i, j, k);
  if (!in_v0(g, c, i, j, k)) return __ldg(r.cur(c) + off);  // u_new not written this step: last value
  const R* row;
  R dv, u;
  if (c == 0) {
    dv = div_x<S>(a, f, i, j, k, t1_at<S>(a, f, i + 1, j, k, 0), t1_at<S>(a, f, i, j, k, 0), t6_at<S>(a, f, i, j, k),
                  t6_at<S>(a, f, i, j - 1, k), t5_at<S>(a, f, i, j, k), t5_at<S>(a, f, i, j, k - 1), row);
    u = f.x(i, j, k);
  } else if (c == 1) {
    dv = div_y<S>(a, f, i, j, k, t6_at<S>(a, f, i, j, k), t6_at<S>(a, f, i - 1, j, k), t1_at<S>(a, f, i, j + 1, k, 1),
                  t1_at<S>(a, f, i, j, k, 1), t4_at<S>(a, f, i, j, k), t4_at<S>(a, f, i, j, k - 1), row);
    u = f.y(i, j, k);
  } else {
    dv = div_z<S>(a, f, i, j, k, t5_at<S>(a, f, i, j, k), t5_at<S>(a, f, i - 1, j, k), t4_at<S>(a, f, i, j, k),
                  t4_at<S>(a, f, i, j - 1, k), t1_at<S>(a, f, i, j, k + 1, 2), t1_at<S>(a, f, i, j, k, 2), row);
    u = f.z(i, j, k);
  }
  R vn, cn;
  return update_value<S>(u, load_pw<S>(r, c, off), dv, row, vn, cn);
}

// final value of a face point: walk z=N, y=N, y=0, x=N (reverse of the
// reference order), evaluate the interior value at the end, apply the faces
// from_out: the interior value of the chain end is read from the new state,
// which the tile pass has already written (separate face pass); otherwise it
// is evaluated here from the input state (fused launch).  The chain end is
// never a face point when ny >= 4, which is when the separate pass is used.
template <class S>
__device__ typename S::R face_value(const StepArgs<typename S::R>& a, const Roles<typename S::R>& r,
                                    const GlobalFetch<typename S::R>& f, int c, int i, int j, int k,
                                    bool from_out) {
  using R = typename S::R;
  const Geo& g = a.g;
  const int xi = ext_x(g, c) - 1, jN = ext_y(g, c) - 1, kz = ext_z(g, c) - 1;
  int ci = i, cj = j, ck = k;
  const bool sz = ck == kz;  // z = N face at (i, j, kz)
  if (sz) ck -= 1;
  const bool syn = cj == jN;  // y = N face at (i, jN, ck)
  const int kyn = ck;
  if (syn) cj -= 1;
  const bool sy0 = cj == 0;  // y = 0 face at (i, 0, ck)
  if (sy0) cj += 1;
  const bool sx = ci == xi;  // x = N face at (xi, cj, ck)
  if (sx) ci -= 1;
  auto U = [&](int ii, int jj, int kk) -> R {
    return c == 0 ? f.x(ii, jj, kk) : (c == 1 ? f.y(ii, jj, kk) : f.z(ii, jj, kk));
  };
  R val = from_out ? r.out(c)[fidx(g, ci, cj, ck)] : v0_global<S>(a, r, f, c, ci, cj, ck);
  if (sx) val = S::abc(c == 0 ? a.abc[0] : a.abc[1], val, U(xi, cj, ck), U(xi - 1, cj, ck));
  if (sy0) val = S::abc(c == 1 ? a.abc[3] : a.abc[2], val, U(i, 0, kyn), U(i, 1, kyn));
  if (syn) val = S::abc(c == 1 ? a.abc[5] : a.abc[4], val, U(i, jN, kyn), U(i, jN - 1, kyn));
  if (sz) val = S::abc(c == 2 ? a.abc[7] : a.abc[6], val, U(i, j, kz), U(i, j, kz - 1));
  return val;
}

// one face point: flattened index -> (component, plane, i, j, k), final value,
// state store and surface record
template <class S>
__device__ __forceinline__ void face_point(const StepArgs<typename S::R>& a, const Roles<typename S::R>& r,
                                           const typename S::R s, const int tt, const int idx, const bool from_out) {
  using R = typename S::R;
  const Geo& g = a.g;
  if (idx >= a.faces.off[12]) return;
  int q = 0;
  while (q < 11 && idx >= a.faces.off[q + 1]) q++;
  const int c = q >> 2, pl = q & 3, rr = idx - a.faces.off[q];
  const int ex = ext_x(g, c), ey = ext_y(g, c), ez = ext_z(g, c);
  int i, j, k;
  if (pl == 0) {  // z = N points that are also on an x / y face (the rest: tile pass)
    k = ez - 1;
    if (rr < ex) { i = rr; j = 0; }
    else if (rr < 2 * ex) { i = rr - ex; j = ey - 1; }
    else { i = ex - 1; j = 1 + rr - 2 * ex; }
  }
  else if (pl == 1) { i = rr / (ez - 1); k = rr - i * (ez - 1); j = ey - 1; }
  else if (pl == 2) { i = rr / (ez - 1); k = rr - i * (ez - 1); j = 0; }
  else { j = rr / (ez - 1); k = rr - j * (ez - 1); j += 1; i = ex - 1; }
  GlobalFetch<R> f{r.cur(0), r.cur(1), r.cur(2), a.mat, a.tab, g, s, a.source_mode};
  R val = a.bc == 1 ? R(0) : face_value<S>(a, r, f, c, i, j, k, from_out);
  long long off = fidx(g, i, j, k);
  store_point<S>(r, c, off, val, R(0), R(0));
  if (c == 2 && k == 0) record(a, tt, i, j, val);
}

// separate face pass: runs after the tile-only step launch on the same stream
template <class S>
__global__ void __launch_bounds__(256) fdtd_face_kernel(const __grid_constant__ StepArgs<typename S::R> a) {
  using R = typename S::R;
  const int tt = __ldg(a.step_base) + a.step_off;
  if (tt >= a.step_end) return;
  const Roles<R> r = roles<S>(a, tt);
  face_point<S>(a, r, (R)__ldg(a.src + tt), tt, blockIdx.x * 256 + threadIdx.x, true);
}

// ---------------------------------------------------------------------------
// TMA + mbarrier helpers (inline PTX)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: false if the phase did not complete within `limit` polls
// (limit <= 0: 2^22 polls, about 0.3 s with the back-off below)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit = 0) {
  if (limit <= 0) limit = 1 << 22;
  for (int it = 0; it < limit; it++) {
    if (mbar_try_wait(bar, parity)) return true;
    if (it > 64) __nanosleep(64);
  }
  return false;
}
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* tm, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(smem_u32(dst)),
      "l"(tm), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, int c0, int c1, int c2,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(tm), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}

// Shared memory of a tile block: mbarriers, the u ring (NSLOT planes of the
// three components with a 1-node halo), the pointwise ring (own points of
// u_old, or of v and the Kahan terms, for the same planes), the material-id
// ring, the stress planes and, last, the material table (its size depends on
// the number of materials, so it is the only variable part).
template <class S, int TJ>
struct SmemPlan {
  using R = typename S::R;
  using TF = TileShape<R, TJ>;
  static constexpr int W = TK + 2, PL = W * (TJ + 2);
  static constexpr int NPW = S::kahan ? 2 : 1;  // pointwise arrays: v and c, or u_old
  static constexpr int PWC = TJ * TK;           // one component of a pointwise tile
  static constexpr int PWS = NPW * 3 * PWC;     // one pointwise slot
  static constexpr size_t BARS = 128;
  static constexpr size_t UR = (size_t)NSLOT * TF::SU * sizeof(R);
  static constexpr size_t PWR = (size_t)NSLOT * PWS * sizeof(R);
  static constexpr size_t MR = (size_t)NSLOT * TF::SM;
  static constexpr size_t TS = ((7 * PL * sizeof(R) + 127) / 128) * 128;
  static constexpr size_t off_u = BARS, off_pw = off_u + UR, off_m = off_pw + PWR, off_t = off_m + MR;
  static constexpr size_t off_tab = off_t + TS;
  static constexpr size_t fixed = off_tab + 128;  // + alignment slack
  static constexpr size_t bytes(int table_rows) { return fixed + (size_t)table_rows * 16 * sizeof(R); }
  static constexpr uint32_t tx_bytes = (uint32_t)(3 * (TJ + 2) * Lay<R>::KW * sizeof(R) + (TJ + 2) * MKW);
  static constexpr uint32_t pw_bytes = (uint32_t)(PWS * sizeof(R));
  static_assert((PWC * sizeof(R)) % 128 == 0 && (TF::SU * sizeof(R)) % 128 == 0, "ring tiles must stay 128-byte aligned");
};

// Rows of one z column a tile-pass thread owns: two for the FP32 velocity
// form at tile heights 8 and 16 (the per-plane work shared by two nodes; 128
// or 256 threads a block), one otherwise.
template <class S, int TJ>
struct RowsPerThread {
  static constexpr int value = (S::kahan && sizeof(typename S::R) == 4 && TJ >= 8) ? 2 : 1;
};

#include "tile_rows.cuh"

// the tile pass of one block: one row per thread or RowsPerThread rows
template <class S, int TJ>
__device__ __forceinline__ bool run_tile(const StepArgs<typename S::R>& a, unsigned char* base,
                                         const Roles<typename S::R>& r, const typename S::R s, const int tt,
                                         const int tid, const int b, const StepArgs<typename S::R>* maps) {
  return tile_block_rows<S, TJ>(a, base, r, s, tt, tid, b, maps);
}

// ---------------------------------------------------------------------------
// the step kernel
// ---------------------------------------------------------------------------
// Resident blocks per SM the register allocation is made for (measured on
// GB300 for the 256x256x128 crystal and the 64-crystal batch).  FP32: tile
// height 4, 6 blocks of 128 threads (up to 85 registers); heights 8 and 16
// (two rows a thread), 4 blocks of 128 or 2 of 256 threads (up to 128
// registers).  FP64: 16 warps per SM.
template <class R, int TJ, bool BATCH = false>
struct MinBlocks {
  static constexpr int value = sizeof(R) == 8 ? (TJ < 16 ? 16 / TJ : 1) : (TJ == 4 ? 6 : (TJ == 8 ? 4 : 2));
};
template <class S, int TJ>
__host__ __device__ constexpr int step_threads() { return TK * TJ / RowsPerThread<S, TJ>::value; }
template <class S, int TJ>
__global__ void __launch_bounds__(step_threads<S, TJ>(), MinBlocks<typename S::R, TJ>::value)
    fdtd_step_kernel(const __grid_constant__ StepArgs<typename S::R> a) {
  using R = typename S::R;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // 128-byte aligned start, derived by pointer arithmetic on the shared array
  // so that every access below stays a shared-memory access (an integer
  // round trip would turn them into generic loads)
  unsigned char* base = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);

  const int tt = __ldg(a.step_base) + a.step_off;
  if (tt >= a.step_end) return;  // a batched instance past its budget
  const Roles<R> r = roles<S>(a, tt);
  const R s = (R)__ldg(a.src + tt);
  const int tid = threadIdx.y * TK + threadIdx.x;

  if ((int)blockIdx.x >= a.n_tile_blocks) {
    // ---------------- face blocks (fused launch) ----------------
    face_point<S>(a, r, s, tt, ((int)blockIdx.x - a.n_tile_blocks) * step_threads<S, TJ>() + tid, false);
    return;
  }

  // ---------------- tile blocks ----------------
  run_tile<S, TJ>(a, base, r, s, tt, tid, blockIdx.x, &a);
}

// ---------------------------------------------------------------------------
// host-side launch helpers (called by the C ABI in api.cu)
// ---------------------------------------------------------------------------
template <class S, int TJ>
static cudaError_t configure_tj() {
  return cudaFuncSetAttribute(fdtd_step_kernel<S, TJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)SmemPlan<S, TJ>::bytes(TAB_ROWS_MAX));
}

template <class S>
cudaError_t configure_step(int tj) {
  switch (tj) {
    case 4: return configure_tj<S, 4>();
    case 8: return configure_tj<S, 8>();
    case 16: return configure_tj<S, 16>();
    default: return cudaErrorInvalidValue;
  }
}

// separate_faces: 0 one fused launch (face points in extra blocks), 1 the tile
// launch then the face launch; 2 only the tile launch and 3 only the face
// launch of the separate form (phono_time_kernels times them apart)
template <class S, int TJ>
static cudaError_t launch_tj(const StepArgs<typename S::R>& a, int separate_faces, cudaStream_t st) {
  const int nfaces = a.faces.off[12];
  constexpr int NT = step_threads<S, TJ>();
  dim3 block(TK, NT / TK);
  // fused: face points handled by extra blocks of the same launch
  dim3 grid(a.n_tile_blocks + (separate_faces ? 0 : (nfaces + NT - 1) / NT));
  if (separate_faces != 3) fdtd_step_kernel<S, TJ><<<grid, block, SmemPlan<S, TJ>::bytes(a.nmat), st>>>(a);
  if ((separate_faces == 1 || separate_faces == 3) && nfaces > 0)
    fdtd_face_kernel<S><<<(nfaces + 255) / 256, 256, 0, st>>>(a);
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_step(const StepArgs<typename S::R>& a, int tj, int separate_faces, cudaStream_t st) {
  switch (tj) {
    case 4: return launch_tj<S, 4>(a, separate_faces, st);
    case 8: return launch_tj<S, 8>(a, separate_faces, st);
    case 16: return launch_tj<S, 16>(a, separate_faces, st);
    default: return cudaErrorInvalidValue;
  }
}

// ---------------------------------------------------------------------------
// batched instances: persistent tile kernel + face kernel + counter update
// ---------------------------------------------------------------------------
template <class S, int TJ>
__global__ void __launch_bounds__(step_threads<S, TJ>(), MinBlocks<typename S::R, TJ, true>::value)
    batch_step_kernel(const __grid_constant__ BatchArgs<typename S::R> ba) {
  using R = typename S::R;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  __shared__ StepArgs<R> sa;  // the current item's instance arguments
  __shared__ int item;
  const int tid = threadIdx.y * TK + threadIdx.x;
  const int n_items = __ldg(ba.counts);
  for (;;) {
    // each block takes items until one past the end; the counter wraps to 0
    // after the last of the n_items + gridDim.x requests
    if (tid == 0) item = (int)atomicInc(ba.ticket, (unsigned)(n_items + gridDim.x - 1));
    __syncthreads();
    const int it = item;
    if (it >= n_items) break;
    const int2 w = ba.items[it];
    const int4* src4 = reinterpret_cast<const int4*>(ba.inst + w.x);
    int4* dst4 = reinterpret_cast<int4*>(&sa);
    for (int q = tid; q < (int)(sizeof(StepArgs<R>) / 16); q += step_threads<S, TJ>()) dst4[q] = src4[q];
    __syncthreads();
    const int tt = *sa.step_base + ba.step_off;
    if (tt < sa.step_end) {
      const Roles<R> r = roles<S>(sa, tt);
      run_tile<S, TJ>(sa, base, r, (R)__ldg(sa.src + tt), tt, tid, w.y, ba.inst + w.x);
    }
    __syncthreads();  // sa and item are rewritten by the next iteration
  }
}

template <class S>
__global__ void __launch_bounds__(256) batch_face_kernel(const __grid_constant__ BatchArgs<typename S::R> ba) {
  using R = typename S::R;
  const int n_fb = __ldg(ba.counts + 1), n_ent = __ldg(ba.counts + 2);
  for (int fb = blockIdx.x; fb < n_fb; fb += gridDim.x) {
    int lo = 0, hi = n_ent - 1;  // last entry whose first block <= fb
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(ba.face_prefix + mid) <= fb) lo = mid;
      else hi = mid - 1;
    }
    const StepArgs<R>& a = ba.inst[__ldg(ba.face_inst + lo)];
    const int tt = *a.step_base + ba.step_off;
    if (tt >= a.step_end) continue;
    const Roles<R> r = roles<S>(a, tt);
    face_point<S>(a, r, (R)__ldg(a.src + tt), tt, (fb - __ldg(ba.face_prefix + lo)) * 256 + threadIdx.x, true);
  }
}

// advance the step counter of every active instance by n, stopping at its budget
template <class R>
__global__ void batch_advance_kernel(const __grid_constant__ BatchArgs<R> ba, int n) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= __ldg(ba.counts + 3)) return;
  const StepArgs<R>& a = ba.inst[__ldg(ba.active + q)];
  int* c = const_cast<int*>(a.step_base);
  *c = min(*c + n, a.step_end);
}

template <class S, int TJ>
static cudaError_t batch_launch_tj(const BatchArgs<typename S::R>& ba, int grid_tiles, int grid_faces,
                                   cudaStream_t st) {
  batch_step_kernel<S, TJ>
      <<<grid_tiles, dim3(TK, step_threads<S, TJ>() / TK), SmemPlan<S, TJ>::bytes(BATCH_TAB_ROWS), st>>>(ba);
  batch_face_kernel<S><<<grid_faces, 256, 0, st>>>(ba);
  return cudaGetLastError();
}

template <class S>
cudaError_t batch_step(const BatchArgs<typename S::R>& ba, int tj, int grid_tiles, int grid_faces, cudaStream_t st) {
  switch (tj) {
    case 4: return batch_launch_tj<S, 4>(ba, grid_tiles, grid_faces, st);
    case 8: return batch_launch_tj<S, 8>(ba, grid_tiles, grid_faces, st);
    case 16: return batch_launch_tj<S, 16>(ba, grid_tiles, grid_faces, st);
    default: return cudaErrorInvalidValue;
  }
}

template <class S, int TJ>
static cudaError_t batch_configure_tj(int* blocks_per_sm) {
  const int smem = (int)SmemPlan<S, TJ>::bytes(BATCH_TAB_ROWS);
  cudaError_t e = cudaFuncSetAttribute(batch_step_kernel<S, TJ>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, batch_step_kernel<S, TJ>, step_threads<S, TJ>(),
                                                       smem);
}

template <class S>
cudaError_t batch_configure(int tj, int* blocks_per_sm) {
  switch (tj) {
    case 4: return batch_configure_tj<S, 4>(blocks_per_sm);
    case 8: return batch_configure_tj<S, 8>(blocks_per_sm);
    case 16: return batch_configure_tj<S, 16>(blocks_per_sm);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t batch_step_any(int precision, const void* ba, int tj, int grid_tiles, int grid_faces, cudaStream_t st) {
  if (precision == 0) return batch_step<F64>(*(const BatchArgs<double>*)ba, tj, grid_tiles, grid_faces, st);
  if (precision == 2) return batch_step<F64V>(*(const BatchArgs<double>*)ba, tj, grid_tiles, grid_faces, st);
  return batch_step<F32K>(*(const BatchArgs<float>*)ba, tj, grid_tiles, grid_faces, st);
}

cudaError_t batch_advance_any(int precision, const void* ba, int n_active_cap, int n, cudaStream_t st) {
  const int blocks = (n_active_cap + 255) / 256;
  if (precision == 1) batch_advance_kernel<float><<<blocks, 256, 0, st>>>(*(const BatchArgs<float>*)ba, n);
  else batch_advance_kernel<double><<<blocks, 256, 0, st>>>(*(const BatchArgs<double>*)ba, n);
  return cudaGetLastError();
}

cudaError_t batch_configure_any(int precision, int tj, int* blocks_per_sm) {
  if (precision == 0) return batch_configure<F64>(tj, blocks_per_sm);
  if (precision == 2) return batch_configure<F64V>(tj, blocks_per_sm);
  return batch_configure<F32K>(tj, blocks_per_sm);
}

// non-template entry points for the C ABI translation unit
cudaError_t configure_step_f64(int tj) { return configure_step<F64>(tj); }
cudaError_t configure_step_f32k(int tj) { return configure_step<F32K>(tj); }
cudaError_t launch_step_f64(const StepArgs<double>& a, int tj, int nf, cudaStream_t st) {
  return launch_step<F64>(a, tj, nf, st);
}
cudaError_t launch_step_f32k(const StepArgs<float>& a, int tj, int nf, cudaStream_t st) {
  return launch_step<F32K>(a, tj, nf, st);
}
cudaError_t configure_step_f64v(int tj) { return configure_step<F64V>(tj); }
cudaError_t launch_step_f64v(const StepArgs<double>& a, int tj, int nf, cudaStream_t st) {
  return launch_step<F64V>(a, tj, nf, st);
}

}  // namespace phono
