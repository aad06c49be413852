// Fused elastic FDTD step for GB300 (sm_103a).
//
// One launch advances one time step of phonomena's staggered-grid solver
// (simulation/base_solver.py:245-266).  The launch has two kinds of blocks:
//
//  * tile blocks: a (TJ x 32) tile of the (y, z) plane marches along x over a
//    segment of planes.  Each iteration loads the next plane of u (3
//    components, 1-node halo) into a 3-plane shared-memory ring, evaluates the
//    six stresses of the current plane once (plus the halo stresses the
//    neighbours need) into shared memory, and writes the new displacement of
//    the plane.  Stresses are never written to global memory.
//
//  * face blocks: one thread per point of the four absorbing faces
//    (x=N, y=0, y=N, z=N; simulation/base_solver.py:540-554).  The reference
//    applies the faces one after another, each reading the plane next to it
//    as left by the earlier faces; the final value of a face point is thus a
//    chain of at most four face formulas ending at the interior value of one
//    point q.  The face thread walks that chain and evaluates q's interior
//    value itself from the input state, so faces need no second pass.
//
// Two arithmetic schemes share this structure:
//  F64  - the reference leapfrog u' = (2u - u_old) + (dt^2/P) * div T with the
//         reference's IEEE operation order (explicit _rn intrinsics, true
//         division), bit-identical to the reference CPU solver.
//  F32K - FP32 velocity form v' = v + (dt/P) div T, u' = u + dt v' with a
//         Kahan-compensated displacement sum; explicit fmaf only.
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
  // normal stresses ((C0*d1)/a + (C1*d2)/b) + (C2*d3)/d   (base_solver.py:329-351)
  __device__ __forceinline__ static void tn(const R* c, R d1, R d2, R d3, R a, R b, R d, R& T1, R& T2, R& T3,
                                            bool want3) {
    T1 = __dadd_rn(__dadd_rn(__ddiv_rn(__dmul_rn(__ldg(c + 0), d1), a), __ddiv_rn(__dmul_rn(__ldg(c + 1), d2), b)),
                   __ddiv_rn(__dmul_rn(__ldg(c + 2), d3), d));
    T2 = __dadd_rn(__dadd_rn(__ddiv_rn(__dmul_rn(__ldg(c + 3), d1), a), __ddiv_rn(__dmul_rn(__ldg(c + 4), d2), b)),
                   __ddiv_rn(__dmul_rn(__ldg(c + 5), d3), d));
    T3 = want3 ? __dadd_rn(__dadd_rn(__ddiv_rn(__dmul_rn(__ldg(c + 6), d1), a),
                                     __ddiv_rn(__dmul_rn(__ldg(c + 7), d2), b)),
                           __ddiv_rn(__dmul_rn(__ldg(c + 8), d3), d))
               : 0.0;
  }
  // shear stress C * (d1/a + d2/b)   (base_solver.py:353-372)
  __device__ __forceinline__ static R ts(R cs, R d1, R a, R d2, R b) {
    return __dmul_rn(cs, __dadd_rn(__ddiv_rn(d1, a), __ddiv_rn(d2, b)));
  }
  // (d1/a + d2/b) + d3/c   (base_solver.py:444-446)
  __device__ __forceinline__ static R div3(R d1, R a, R d2, R b, R d3, R c) {
    return __dadd_rn(__dadd_rn(__ddiv_rn(d1, a), __ddiv_rn(d2, b)), __ddiv_rn(d3, c));
  }
  // uz z=0 row as written at base_solver.py:516: ((d1/a + d2/b) + T3[..,1]) - T3[..,0]/fdz
  // with T3[..,0] == +0, so the last subtraction is exact and dropped.
  __device__ __forceinline__ static R div_surf_ref(R d1, R a, R d2, R b, R t31) {
    return __dadd_rn(__dadd_rn(__ddiv_rn(d1, a), __ddiv_rn(d2, b)), t31);
  }
  // u[b-+1] + c * (u_new[b-+1] - u[b])   (base_solver.py:540-554)
  __device__ __forceinline__ static R abc(R coef, R nbr_new, R self_old, R nbr_old) {
    return __dadd_rn(nbr_old, __dmul_rn(coef, __dsub_rn(nbr_new, self_old)));
  }
  // (2u - u_old) + (dt^2/P) * div   (base_solver.py:441-443)
  __device__ __forceinline__ static R leap(R u, R uold, R dt2p, R dv) {
    return __dadd_rn(__dsub_rn(__dmul_rn(2.0, u), uold), __dmul_rn(dt2p, dv));
  }
};

struct F32K {
  using R = float;
  static constexpr bool kahan = true;
  __device__ __forceinline__ static R sub(R a, R b) { return __fsub_rn(a, b); }
  __device__ __forceinline__ static void tn(const R* c, R d1, R d2, R d3, R a, R b, R d, R& T1, R& T2, R& T3,
                                            bool want3) {
    R e1 = __fmul_rn(d1, a), e2 = __fmul_rn(d2, b), e3 = __fmul_rn(d3, d);
    T1 = __fmaf_rn(__ldg(c + 0), e1, __fmaf_rn(__ldg(c + 1), e2, __fmul_rn(__ldg(c + 2), e3)));
    T2 = __fmaf_rn(__ldg(c + 3), e1, __fmaf_rn(__ldg(c + 4), e2, __fmul_rn(__ldg(c + 5), e3)));
    T3 = want3 ? __fmaf_rn(__ldg(c + 6), e1, __fmaf_rn(__ldg(c + 7), e2, __fmul_rn(__ldg(c + 8), e3))) : 0.0f;
  }
  __device__ __forceinline__ static R ts(R cs, R d1, R a, R d2, R b) {
    return __fmul_rn(cs, __fmaf_rn(d1, a, __fmul_rn(d2, b)));
  }
  __device__ __forceinline__ static R div3(R d1, R a, R d2, R b, R d3, R c) {
    return __fmaf_rn(d1, a, __fmaf_rn(d2, b, __fmul_rn(d3, c)));
  }
  __device__ __forceinline__ static R div_surf_ref(R d1, R a, R d2, R b, R t31) {
    return __fadd_rn(__fmaf_rn(d1, a, __fmul_rn(d2, b)), t31);
  }
  __device__ __forceinline__ static R abc(R coef, R nbr_new, R self_old, R nbr_old) {
    return __fmaf_rn(coef, __fsub_rn(nbr_new, self_old), nbr_old);
  }
};

// ---------------------------------------------------------------------------
// addressing
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long fidx(const Geo& g, int i, int j, int k) {
  return g.o0 + (long long)i * g.sx + (long long)j * g.sy + k;
}
template <class R>
__device__ __forceinline__ const R* mrow(const StepArgs<R>& a, int i, int j, int k) {
  int m = __ldg(a.mat + a.g.mo0 + (long long)i * a.g.msx + (long long)j * a.g.msy + k);
  return a.tab + m * 16;
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
// stress at a point, given a displacement fetcher F (x/y/z(i,j,k) -> R)
// zero wherever the reference never writes the stress array
// ---------------------------------------------------------------------------
template <class S, class F>
__device__ __forceinline__ void t123_at(const StepArgs<typename S::R>& a, const F& f, int i, int j, int k,
                                        typename S::R& T1, typename S::R& T2, typename S::R& T3) {
  using R = typename S::R;
  const Geo& g = a.g;
  if (i < 1 || i > g.nx - 2 || j < 1 || j > g.ny - 2 || k < 0 || k > g.nz - 2) {
    T1 = T2 = T3 = R(0);
    return;
  }
  const R* c = mrow(a, i, j, k);
  R d1 = S::sub(f.x(i, j, k), f.x(i - 1, j, k));
  R d2 = S::sub(f.y(i, j, k), f.y(i, j - 1, k));
  if (k == 0) {  // base_solver.py:408-418 (uz - 0, scalar spacings, T3 = 0)
    R d3 = f.z(i, j, 0);
    S::tn(c, d1, d2, d3, a.sp.sdx0, a.sp.sdy0, a.sp.sdz0, T1, T2, T3, false);
  } else {
    R d3 = S::sub(f.z(i, j, k), f.z(i, j, k - 1));
    S::tn(c, d1, d2, d3, __ldg(a.sp.sdx + i - 1), __ldg(a.sp.sdy + j - 1), __ldg(a.sp.sdz + k - 1), T1, T2, T3,
          true);
  }
}

template <class S, class F>
__device__ __forceinline__ typename S::R t4_at(const StepArgs<typename S::R>& a, const F& f, int i, int j, int k) {
  using R = typename S::R;
  const Geo& g = a.g;
  if (i < 1 || i > g.nx - 2 || j < 0 || j > g.ny - 2 || k < 0 || k > g.nz - 2) return R(0);
  if (k == 0)  // base_solver.py:420-423
    return S::ts(__ldg(mrow(a, i, j + 1, 0) + 9), S::sub(f.y(i, j, 1), f.y(i, j, 0)), a.sp.fdy0,
                 S::sub(f.z(i, j + 1, 0), f.z(i, j, 0)), a.sp.fdz0);
  return S::ts(__ldg(mrow(a, i, j + 1, k + 1) + 9), S::sub(f.y(i, j, k + 1), f.y(i, j, k)), __ldg(a.sp.fdz + k),
               S::sub(f.z(i, j + 1, k), f.z(i, j, k)), __ldg(a.sp.fdy + j));
}

template <class S, class F>
__device__ __forceinline__ typename S::R t5_at(const StepArgs<typename S::R>& a, const F& f, int i, int j, int k) {
  using R = typename S::R;
  const Geo& g = a.g;
  if (i < 0 || i > g.nx - 2 || j < 1 || j > g.ny - 2 || k < 0 || k > g.nz - 2) return R(0);
  if (k == 0)  // base_solver.py:425-428
    return S::ts(__ldg(mrow(a, i + 1, j, 0) + 10), S::sub(f.x(i, j, 1), f.x(i, j, 0)), a.sp.fdx0,
                 S::sub(f.z(i + 1, j, 0), f.z(i, j, 0)), a.sp.fdz0);
  return S::ts(__ldg(mrow(a, i + 1, j, k + 1) + 10), S::sub(f.x(i, j, k + 1), f.x(i, j, k)), __ldg(a.sp.fdz + k),
               S::sub(f.z(i + 1, j, k), f.z(i, j, k)), __ldg(a.sp.fdx + i));
}

template <class S, class F>
__device__ __forceinline__ typename S::R t6_at(const StepArgs<typename S::R>& a, const F& f, int i, int j, int k) {
  using R = typename S::R;
  const Geo& g = a.g;
  if (i < 0 || i > g.nx - 2 || j < 0 || j > g.ny - 2 || k < 0 || k > g.nz - 2) return R(0);
  if (k == 0)  // base_solver.py:430-433
    return S::ts(__ldg(mrow(a, i + 1, j + 1, 0) + 11), S::sub(f.x(i, j + 1, 0), f.x(i, j, 0)), a.sp.fdx0,
                 S::sub(f.y(i + 1, j, 0), f.y(i, j, 0)), a.sp.fdz0);
  return S::ts(__ldg(mrow(a, i + 1, j + 1, k) + 11), S::sub(f.x(i, j + 1, k), f.x(i, j, k)), __ldg(a.sp.fdy + j),
               S::sub(f.y(i + 1, j, k), f.y(i, j, k)), __ldg(a.sp.fdx + i));
}

// divergence terms of the three components (base_solver.py:441-463,495-516)
// and the material row whose density applies
template <class S>
__device__ __forceinline__ typename S::R div_x(const StepArgs<typename S::R>& a, int i, int j, int k,
                                               typename S::R t1p, typename S::R t1m, typename S::R t6a,
                                               typename S::R t6b, typename S::R t5a, typename S::R t5b,
                                               const typename S::R*& row) {
  if (k == 0) {
    row = mrow(a, i + 1, j, 0);
    return S::div3(S::sub(t1p, t1m), a.sp.fdx0, S::sub(t6a, t6b), a.sp.sdy0, t5a, a.sp.sdz0);
  }
  row = mrow(a, i + 1, j, k);
  return S::div3(S::sub(t1p, t1m), __ldg(a.sp.fdx + i), S::sub(t6a, t6b), __ldg(a.sp.sdy + j - 1),
                 S::sub(t5a, t5b), __ldg(a.sp.sdz + k - 1));
}
template <class S>
__device__ __forceinline__ typename S::R div_y(const StepArgs<typename S::R>& a, int i, int j, int k,
                                               typename S::R t6a, typename S::R t6b, typename S::R t2p,
                                               typename S::R t2m, typename S::R t4a, typename S::R t4b,
                                               const typename S::R*& row) {
  if (k == 0) {
    row = mrow(a, i, j + 1, 0);
    return S::div3(S::sub(t6a, t6b), a.sp.sdx0, S::sub(t2p, t2m), a.sp.fdy0, t4a, a.sp.sdz0);
  }
  row = mrow(a, i, j + 1, k);
  return S::div3(S::sub(t6a, t6b), __ldg(a.sp.sdx + i - 1), S::sub(t2p, t2m), __ldg(a.sp.fdy + j),
                 S::sub(t4a, t4b), __ldg(a.sp.sdz + k - 1));
}
template <class S>
__device__ __forceinline__ typename S::R div_z(const StepArgs<typename S::R>& a, int i, int j, int k,
                                               typename S::R t5a, typename S::R t5b, typename S::R t4a,
                                               typename S::R t4b, typename S::R t3p, typename S::R t3m,
                                               const typename S::R*& row) {
  if (k == 0) {
    row = mrow(a, i, j, 0);  // density at z index 0 (base_solver.py:513)
    if (a.surface_mode == 0) return S::div_surf_ref(S::sub(t5a, t5b), a.sp.sdx0, S::sub(t4a, t4b), a.sp.sdy0, t3p);
    return S::div3(S::sub(t5a, t5b), a.sp.sdx0, S::sub(t4a, t4b), a.sp.sdy0, t3p, a.sp.fdz0);
  }
  row = mrow(a, i, j, k + 1);
  return S::div3(S::sub(t5a, t5b), __ldg(a.sp.sdx + i - 1), S::sub(t4a, t4b), __ldg(a.sp.sdy + j - 1),
                 S::sub(t3p, t3m), __ldg(a.sp.fdz + k));
}

// state roles of global step tt
template <class R>
struct Roles {
  const R* cur[3];  // u at step tt (before the source overwrite)
  const R* old[3];  // F64: u at tt-1
  R* out[3];        // u at tt+1
  const R* vin[3];
  const R* cin[3];
  R* vout[3];
  R* cout[3];
};

template <class S>
__device__ __forceinline__ Roles<typename S::R> roles(const StepArgs<typename S::R>& a, int tt) {
  Roles<typename S::R> r;
  if (!S::kahan) {
    int ro = tt % 3, rc = (tt + 1) % 3, rn = (tt + 2) % 3;
    for (int c = 0; c < 3; c++) {
      r.old[c] = a.u[ro][c];
      r.cur[c] = a.u[rc][c];
      r.out[c] = a.u[rn][c];
      r.vin[c] = r.cin[c] = nullptr;
      r.vout[c] = r.cout[c] = nullptr;
    }
  } else {
    int bi = tt & 1, bo = bi ^ 1;
    for (int c = 0; c < 3; c++) {
      r.cur[c] = a.u[bi][c];
      r.old[c] = nullptr;
      r.out[c] = a.u[bo][c];
      r.vin[c] = a.v[bi][c];
      r.cin[c] = a.c[bi][c];
      r.vout[c] = a.v[bo][c];
      r.cout[c] = a.c[bo][c];
    }
  }
  return r;
}

// new state of one V0 point: F64 leapfrog / F32K Kahan velocity update;
// returns the new u and stores it (plus v, c)
template <class S>
__device__ __forceinline__ typename S::R update_point(const StepArgs<typename S::R>& a,
                                                      const Roles<typename S::R>& r, int c, long long off,
                                                      typename S::R u, typename S::R dv,
                                                      const typename S::R* row, bool store) {
  using R = typename S::R;
  if constexpr (!S::kahan) {
    R un = S::leap(u, __ldg(r.old[c] + off), __ldg(row + 12), dv);
    if (store) r.out[c][off] = un;
    return un;
  } else {
    R v = __ldg(r.vin[c] + off), cm = __ldg(r.cin[c] + off);
    R vn = __fmaf_rn(__ldg(row + 12), dv, v);
    R y = __fmaf_rn(__ldg(row + 14), vn, -cm);  // row[14] = dt
    R t = __fadd_rn(u, y);
    if (store) {
      r.cout[c][off] = __fsub_rn(__fsub_rn(t, u), y);
      r.vout[c][off] = vn;
      r.out[c][off] = t;
    }
    return t;
  }
}

template <class S>
__device__ __forceinline__ void store_stale(const Roles<typename S::R>& r, int c, long long off) {
  r.out[c][off] = __ldg(r.cur[c] + off);
  if constexpr (S::kahan) {
    r.vout[c][off] = __ldg(r.vin[c] + off);
    r.cout[c][off] = __ldg(r.cin[c] + off);
  }
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
  Geo g;
  R s;
  int wall;
  __device__ __forceinline__ R x(int i, int j, int k) const { return __ldg(ux + fidx(g, i, j, k)); }
  __device__ __forceinline__ R y(int i, int j, int k) const { return __ldg(uy + fidx(g, i, j, k)); }
  __device__ __forceinline__ R z(int i, int j, int k) const {
    if (i == 0 && (wall || k == 0)) return s;  // source overwrite (base_solver.py:251)
    return __ldg(uz + fidx(g, i, j, k));
  }
};

template <class R, int TJ>
struct TileFetch {
  static constexpr int W = TK + 2, PL = W * (TJ + 2);
  const R* su;  // [3 slots][3 comps][PL]
  int j0, k0;
  __device__ __forceinline__ int loc(int i, int j, int k) const {
    return (((i + 3) % 3) * 3) * PL + (j - j0 + 1) * W + (k - k0 + 1);
  }
  __device__ __forceinline__ R x(int i, int j, int k) const { return su[loc(i, j, k)]; }
  __device__ __forceinline__ R y(int i, int j, int k) const { return su[loc(i, j, k) + PL]; }
  __device__ __forceinline__ R z(int i, int j, int k) const { return su[loc(i, j, k) + 2 * PL]; }
};

// interior (V0) value of u_new at a point, evaluated from global memory
template <class S>
__device__ typename S::R v0_global(const StepArgs<typename S::R>& a, const Roles<typename S::R>& r,
                                   const GlobalFetch<typename S::R>& f, int c, int i, int j, int k) {
  using R = typename S::R;
  const Geo& g = a.g;
  long long off = fidx(g, i, j, k);
  if (!in_v0(g, c, i, j, k)) return __ldg(r.cur[c] + off);  // u_new not written this step: last value
  const R* row;
  R dv, u;
  if (c == 0) {
    R t1p, t1m, d0, d1;
    t123_at<S>(a, f, i + 1, j, k, t1p, d0, d1);
    t123_at<S>(a, f, i, j, k, t1m, d0, d1);
    dv = div_x<S>(a, i, j, k, t1p, t1m, t6_at<S>(a, f, i, j, k), t6_at<S>(a, f, i, j - 1, k),
                  t5_at<S>(a, f, i, j, k), t5_at<S>(a, f, i, j, k - 1), row);
    u = f.x(i, j, k);
  } else if (c == 1) {
    R t2p, t2m, d0, d1;
    t123_at<S>(a, f, i, j + 1, k, d0, t2p, d1);
    t123_at<S>(a, f, i, j, k, d0, t2m, d1);
    dv = div_y<S>(a, i, j, k, t6_at<S>(a, f, i, j, k), t6_at<S>(a, f, i - 1, j, k), t2p, t2m,
                  t4_at<S>(a, f, i, j, k), t4_at<S>(a, f, i, j, k - 1), row);
    u = f.y(i, j, k);
  } else {
    R t3p, t3m, d0, d1;
    t123_at<S>(a, f, i, j, k + 1, d0, d1, t3p);
    t123_at<S>(a, f, i, j, k, d0, d1, t3m);
    dv = div_z<S>(a, i, j, k, t5_at<S>(a, f, i, j, k), t5_at<S>(a, f, i - 1, j, k), t4_at<S>(a, f, i, j, k),
                  t4_at<S>(a, f, i, j - 1, k), t3p, t3m, row);
    u = f.z(i, j, k);
  }
  return update_point<S>(a, r, c, off, u, dv, row, false);
}

// final value of a face point: walk z=N, y=N, y=0, x=N (reverse of the
// reference order), evaluate the interior value at the end, apply the faces
template <class S>
__device__ typename S::R face_value(const StepArgs<typename S::R>& a, const Roles<typename S::R>& r,
                                    const GlobalFetch<typename S::R>& f, int c, int i, int j, int k) {
  using R = typename S::R;
  const Geo& g = a.g;
  const int xi = ext_x(g, c) - 1, jN = ext_y(g, c) - 1, kz = ext_z(g, c) - 1;
  int st[4], pi[4], pj[4], pk[4], n = 0;
  int ci = i, cj = j, ck = k;
  if (ck == kz) { st[n] = 3; pi[n] = ci; pj[n] = cj; pk[n] = ck; n++; ck -= 1; }
  if (cj == jN) { st[n] = 2; pi[n] = ci; pj[n] = cj; pk[n] = ck; n++; cj -= 1; }
  if (cj == 0)  { st[n] = 1; pi[n] = ci; pj[n] = cj; pk[n] = ck; n++; cj += 1; }
  if (ci == xi) { st[n] = 0; pi[n] = ci; pj[n] = cj; pk[n] = ck; n++; ci -= 1; }
  R val = v0_global<S>(a, r, f, c, ci, cj, ck);
  auto U = [&](int ii, int jj, int kk) -> R {
    return c == 0 ? f.x(ii, jj, kk) : (c == 1 ? f.y(ii, jj, kk) : f.z(ii, jj, kk));
  };
  for (int q = n - 1; q >= 0; q--) {
    int bi = pi[q], bj = pj[q], bk = pk[q];
    R coef;
    int ni = bi, nj = bj, nk = bk;
    switch (st[q]) {
      case 0: coef = c == 0 ? a.abc[0] : a.abc[1]; ni = bi - 1; break;      // x = N: clx / ctx
      case 1: coef = c == 1 ? a.abc[3] : a.abc[2]; nj = bj + 1; break;      // y = 0: cly / cty
      case 2: coef = c == 1 ? a.abc[5] : a.abc[4]; nj = bj - 1; break;      // y = N
      default: coef = c == 2 ? a.abc[7] : a.abc[6]; nk = bk - 1; break;     // z = N: clz / ctz
    }
    val = S::abc(coef, val, U(bi, bj, bk), U(ni, nj, nk));
  }
  return val;
}

// ---------------------------------------------------------------------------
// the step kernel
// ---------------------------------------------------------------------------
template <class S, int TJ>
__global__ void __launch_bounds__(TK * TJ) fdtd_step_kernel(const StepArgs<typename S::R> a) {
  using R = typename S::R;
  constexpr int NT = TK * TJ;
  constexpr int W = TK + 2, PL = W * (TJ + 2);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* su = reinterpret_cast<R*>(smem_raw);  // [3][3][PL]
  R* sT2 = su + 9 * PL;
  R* sT3 = sT2 + PL;
  R* sT4 = sT3 + PL;
  R* sT5 = sT4 + PL;  // [2][PL]
  R* sT6 = sT5 + 2 * PL;  // [2][PL]

  const Geo& g = a.g;
  const int tt = __ldg(a.step_base) + a.step_off;
  const Roles<R> r = roles<S>(a, tt);
  const R s = (R)__ldg(a.src + tt);
  const int tid = threadIdx.y * TK + threadIdx.x;

  if ((int)blockIdx.x >= a.n_tile_blocks) {
    // ---------------- face blocks ----------------
    int idx = ((int)blockIdx.x - a.n_tile_blocks) * NT + tid;
    if (idx >= a.faces.off[12]) return;
    int q = 0;
    while (q < 11 && idx >= a.faces.off[q + 1]) q++;
    const int c = q >> 2, pl = q & 3, rr = idx - a.faces.off[q];
    const int ex = ext_x(g, c), ey = ext_y(g, c), ez = ext_z(g, c);
    int i, j, k;
    if (pl == 0) { i = rr / ey; j = rr - i * ey; k = ez - 1; }
    else if (pl == 1) { i = rr / (ez - 1); k = rr - i * (ez - 1); j = ey - 1; }
    else if (pl == 2) { i = rr / (ez - 1); k = rr - i * (ez - 1); j = 0; }
    else { j = rr / (ez - 1); k = rr - j * (ez - 1); j += 1; i = ex - 1; }
    GlobalFetch<R> f{r.cur[0], r.cur[1], r.cur[2], g, s, a.source_mode};
    R val = a.bc == 1 ? R(0) : face_value<S>(a, r, f, c, i, j, k);
    long long off = fidx(g, i, j, k);
    r.out[c][off] = val;
    if constexpr (S::kahan) {
      r.vout[c][off] = R(0);
      r.cout[c][off] = R(0);
    }
    if (c == 2 && k == 0) record(a, tt, i, j, val);
    return;
  }

  // ---------------- tile blocks ----------------
  const int b = blockIdx.x;
  const int kt = b % a.ntk;
  const int rest = b / a.ntk;
  const int jt = rest % a.ntj;
  const int seg = rest / a.ntj;
  const int j0 = jt * TJ, k0 = kt * TK;
  const int ib = seg * a.xseg;
  const int ie = min(ib + a.xseg, g.nx - 1);
  const int j = j0 + threadIdx.y, k = k0 + threadIdx.x;
  const bool active = (j < g.ny - 1) && (k < g.nz - 1);
  const int L = (threadIdx.y + 1) * W + threadIdx.x + 1;
  TileFetch<R, TJ> f{su, j0, k0};

  auto load_plane = [&](int i) {
    R* dst = su + ((i + 3) % 3) * 3 * PL;
    const bool iv = (i >= -1 && i <= g.nx);
    for (int qq = tid; qq < PL; qq += NT) {
      int rr = qq / W, cc = qq - rr * W;
      int gj = j0 - 1 + rr, gk = k0 - 1 + cc;
      R vx = 0, vy = 0, vz = 0;
      if (iv && gj <= g.ny && gk <= g.nz) {
        long long off = fidx(g, i, gj, gk);
        vx = __ldg(r.cur[0] + off);
        vy = __ldg(r.cur[1] + off);
        vz = (i == 0 && (a.source_mode == 1 || gk == 0)) ? s : __ldg(r.cur[2] + off);
      }
      dst[qq] = vx;
      dst[qq + PL] = vy;
      dst[qq + 2 * PL] = vz;
    }
  };

  // prologue: planes ib-1, ib; own T5, T6 at ib-1
  load_plane(ib - 1);
  load_plane(ib);
  __syncthreads();
  R t5m = t5_at<S>(a, f, ib - 1, j, k);
  R t6m = t6_at<S>(a, f, ib - 1, j, k);
  R t1m = 0, uxm = 0;

  for (int i = ib; i <= ie; i++) {
    load_plane(i + 1);
    __syncthreads();
    const int p = i & 1;
    // own stresses at plane i
    R t1c, t2c, t3c;
    t123_at<S>(a, f, i, j, k, t1c, t2c, t3c);
    R t4c = t4_at<S>(a, f, i, j, k);
    R t5c = t5_at<S>(a, f, i, j, k);
    R t6c = t6_at<S>(a, f, i, j, k);
    sT2[L] = t2c;
    sT3[L] = t3c;
    sT4[L] = t4c;
    sT5[p * PL + L] = t5c;
    sT6[p * PL + L] = t6c;
    // halo stresses the neighbours need: T2 row j0+TJ, T6/T4 row j0-1,
    // T3 column k0+TK, T4/T5 column k0-1
    for (int qq = tid; qq < 3 * TK + 3 * TJ; qq += NT) {
      if (qq < TK) {
        int kk = k0 + qq;
        R d0, d1, t2;
        t123_at<S>(a, f, i, j0 + TJ, kk, d0, t2, d1);
        sT2[(TJ + 1) * W + qq + 1] = t2;
      } else if (qq < 2 * TK) {
        int kk = k0 + qq - TK;
        sT6[p * PL + (qq - TK) + 1] = t6_at<S>(a, f, i, j0 - 1, kk);
      } else if (qq < 3 * TK) {
        int kk = k0 + qq - 2 * TK;
        sT4[(qq - 2 * TK) + 1] = t4_at<S>(a, f, i, j0 - 1, kk);
      } else {
        int w = qq - 3 * TK;
        int which = w / TJ, jl = w - which * TJ;
        int jj = j0 + jl;
        if (which == 0) {
          R d0, d1, t3;
          t123_at<S>(a, f, i, jj, k0 + TK, d0, d1, t3);
          sT3[(jl + 1) * W + TK + 1] = t3;
        } else if (which == 1) {
          sT4[(jl + 1) * W] = t4_at<S>(a, f, i, jj, k0 - 1);
        } else {
          sT5[p * PL + (jl + 1) * W] = t5_at<S>(a, f, i, jj, k0 - 1);
        }
      }
    }
    const R uxc = f.x(i, j, k), uyc = f.y(i, j, k), uzc = f.z(i, j, k);
    __syncthreads();
    if (active) {
      if (i < ie) {
        // uy_new(i, j, k)
        long long off = fidx(g, i, j, k);
        if (!on_face(g, 1, i, j, k)) {
          if (in_v0(g, 1, i, j, k)) {
            const R* row;
            R dv = div_y<S>(a, i, j, k, t6c, t6m, sT2[L + W], t2c, t4c, sT4[L - 1], row);
            update_point<S>(a, r, 1, off, uyc, dv, row, true);
          } else {
            store_stale<S>(r, 1, off);
          }
        }
        // uz_new(i, j, k)
        if (!on_face(g, 2, i, j, k)) {
          R val;
          if (in_v0(g, 2, i, j, k)) {
            const R* row;
            R dv = div_z<S>(a, i, j, k, t5c, t5m, t4c, sT4[L - W], sT3[L + 1], t3c, row);
            val = update_point<S>(a, r, 2, off, uzc, dv, row, true);
          } else {
            store_stale<S>(r, 2, off);
            val = __ldg(r.cur[2] + off);
          }
          if (k == 0) record(a, tt, i, j, val);
        }
      }
      if (i > ib) {
        // ux_new(i-1, j, k)
        const int im = i - 1;
        long long off = fidx(g, im, j, k);
        if (!on_face(g, 0, im, j, k)) {
          if (in_v0(g, 0, im, j, k)) {
            const int pm = p ^ 1;
            const R* row;
            R dv = div_x<S>(a, im, j, k, t1c, t1m, sT6[pm * PL + L], sT6[pm * PL + L - W], sT5[pm * PL + L],
                            sT5[pm * PL + L - 1], row);
            update_point<S>(a, r, 0, off, uxm, dv, row, true);
          } else {
            store_stale<S>(r, 0, off);
          }
        }
      }
    }
    t1m = t1c;
    t5m = t5c;
    t6m = t6c;
    uxm = uxc;
  }
}

// ---------------------------------------------------------------------------
// host-side launch helpers (called by the C ABI in api.cu)
// ---------------------------------------------------------------------------
template <class R>
size_t step_smem_bytes(int tj) {
  int PL = (TK + 2) * (tj + 2);
  return sizeof(R) * (size_t)PL * (9 + 3 + 4);
}

template <class S, int TJ>
static cudaError_t configure_tj() {
  return cudaFuncSetAttribute(fdtd_step_kernel<S, TJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)step_smem_bytes<typename S::R>(TJ));
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

template <class S, int TJ>
static cudaError_t launch_tj(const StepArgs<typename S::R>& a, int n_face_blocks, cudaStream_t st) {
  dim3 block(TK, TJ);
  dim3 grid(a.n_tile_blocks + n_face_blocks);
  fdtd_step_kernel<S, TJ><<<grid, block, step_smem_bytes<typename S::R>(TJ), st>>>(a);
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_step(const StepArgs<typename S::R>& a, int tj, int n_face_blocks, cudaStream_t st) {
  switch (tj) {
    case 4: return launch_tj<S, 4>(a, n_face_blocks, st);
    case 8: return launch_tj<S, 8>(a, n_face_blocks, st);
    case 16: return launch_tj<S, 16>(a, n_face_blocks, st);
    default: return cudaErrorInvalidValue;
  }
}

template cudaError_t configure_step<F64>(int);
template cudaError_t configure_step<F32K>(int);
template cudaError_t launch_step<F64>(const StepArgs<double>&, int, int, cudaStream_t);
template cudaError_t launch_step<F32K>(const StepArgs<float>&, int, int, cudaStream_t);
template size_t step_smem_bytes<double>(int);
template size_t step_smem_bytes<float>(int);

}  // namespace phono

// non-template entry points for the C ABI translation unit
namespace phono {
cudaError_t configure_step_f64(int tj) { return configure_step<F64>(tj); }
cudaError_t configure_step_f32k(int tj) { return configure_step<F32K>(tj); }
cudaError_t launch_step_f64(const StepArgs<double>& a, int tj, int nf, cudaStream_t st) {
  return launch_step<F64>(a, tj, nf, st);
}
cudaError_t launch_step_f32k(const StepArgs<float>& a, int tj, int nf, cudaStream_t st) {
  return launch_step<F32K>(a, tj, nf, st);
}
}  // namespace phono
