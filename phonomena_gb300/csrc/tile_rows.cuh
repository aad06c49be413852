// Tile pass of the fused step kernel (included by fdtd_step.cu).
//
// A block owns a (TJ x 32) tile of the (y, z) plane and marches along x over
// planes [ib, ie).  Planes of u (3 components, 1-node halo), material ids and
// the pointwise state of the own points (u_old, or v and the Kahan terms)
// arrive by TMA in a 4-slot ring.  A thread owns JR rows of one z column
// (rows j0 + ty*JR .. + JR-1; JR = RowsPerThread: 2 for FP32 at tile heights
// 8 and 16, else 1), so the per-plane work that does not depend on the row
// (ring waits, barriers, slot addresses, x spacings, the plane's range tests)
// is shared by JR nodes.  Every smem access uses offsets fixed per thread
// and row (own position Lu / Lm, neighbours at constant distance), the range
// predicates of the reference's slices are split into per-row (j, k) and
// per-plane (i) parts computed once, ring values and material ids are carried
// from plane to plane, and the per-axis spacings live in registers, so the
// inner loop is the stencil arithmetic plus shared-memory traffic.  The
// arithmetic goes through the same scheme primitives (tn1, ts, div3,
// update_value) as the face path, operation for operation.
// Included inside namespace phono, after SmemPlan and the scheme primitives.
#pragma once

template <class S, int TJ>
__device__ __forceinline__ bool tile_block_rows(const StepArgs<typename S::R>& a, unsigned char* base,
                                           const Roles<typename S::R>& r, const typename S::R s, const int tt,
                                           const int tid, const int b, const StepArgs<typename S::R>* maps) {
  using R = typename S::R;
  using P = SmemPlan<S, TJ>;
  using TF = TileShape<R, TJ>;
  constexpr int JR = RowsPerThread<S, TJ>::value;
  constexpr int NT = TK * TJ / JR;
  constexpr int W = P::W, PL = P::PL;
  constexpr int KW = TF::KW, KB = TF::KB, CW = TF::CW, SU = TF::SU, SM = TF::SM;
  constexpr int XO = 0, YO = CW, ZO = 2 * CW;  // component offsets inside a ring slot

  uint64_t* bars = reinterpret_cast<uint64_t*>(base);
  R* stab = reinterpret_cast<R*>(base + P::off_tab);
  R* uring = reinterpret_cast<R*>(base + P::off_u);
  R* pwring = reinterpret_cast<R*>(base + P::off_pw);
  uint8_t* mring = reinterpret_cast<uint8_t*>(base + P::off_m);
  R* sT2 = reinterpret_cast<R*>(base + P::off_t);
  R* sT3 = sT2 + PL;
  R* sT4 = sT3 + PL;
  R* sT5 = sT4 + PL;      // [2][PL]
  R* sT6 = sT5 + 2 * PL;  // [2][PL]

  const Geo& g = a.g;
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const int kt = b % a.ntk;
  const int rest = b / a.ntk;
  const int jt = rest % a.ntj;
  const int seg = rest / a.ntj;
  const int j0 = jt * TJ, k0 = kt * TK;
  const int ib = a.nseg <= SEG_TABLE ? a.seg_start[seg] : seg * a.xseg;
  const int ie = a.nseg <= SEG_TABLE ? a.seg_start[seg + 1] : min(ib + a.xseg, nx - 1);
  const int ibase = ib - 1;
  const int plast = ie + 1;  // last plane the segment reads
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int jb = j0 + ty * JR, k = k0 + tx;  // first own row, own column
  const int L = (ty * JR + 1) * W + tx + 1;    // own entry of the stress planes (row r: + r*W)
  const int Lu = (ty * JR + 1) * KW + tx + KB;  // own entry of a u component tile (row r: + r*KW)
  const int Lm = (ty * JR + 1) * MKW + tx + MKOFF;
  const int Lp = ty * JR * TK + tx;            // own entry of a pointwise component tile (row r: + r*TK)

  // the whole material table (nmat <= 256 rows) is staged in shared memory
  for (int q = tid; q < a.nmat * 16; q += NT) stab[q] = __ldg(a.tab + q);
  const R* tab = stab;

  // -------- per-thread and per-row constants (own positions) --------
  // stress ranges of the reference (base_solver.py:329-372, 408-433)
  const bool k_in = k <= nz - 2;  // all six stresses need k <= nz-2
  const bool kz = k == 0;         // traction-free row
  const R sdz_m = k >= 1 && k <= nz - 2 ? __ldg(a.sp.sdz + k - 1) : R(1);
  const R fdz_k = k <= nz - 2 ? __ldg(a.sp.fdz + k) : R(1);
  // spacings as used by the z = 0 row or the interior (the x ones are per plane)
  const R t123_d = kz ? a.sp.sdz0 : sdz_m;  // T1..T3 z; uy and ux z-divergence
  const R uz_c = kz ? (a.surface_mode == 0 ? R(1) : a.sp.fdz0) : fdz_k;
  bool j_n[JR], j_s[JR], own_y[JR], own_z[JR], own_x[JR];
  R sb[JR], fdy_j[JR], uy_b[JR];
  #pragma unroll
  for (int q = 0; q < JR; q++) {
    const int j = jb + q;
    const bool active = (j < ny - 1) && k_in;
    j_n[q] = j >= 1 && j <= ny - 2;  // T1..T3, T5: j in [1, ny-2]
    j_s[q] = j <= ny - 2;            // T4, T6: j in [0, ny-2]
    const R sdy_m = j_n[q] ? __ldg(a.sp.sdy + j - 1) : R(1);
    fdy_j[q] = j_s[q] ? __ldg(a.sp.fdy + j) : R(1);
    sb[q] = kz ? a.sp.sdy0 : sdy_m;  // T1..T3 y; uz and ux y-divergence
    uy_b[q] = kz ? a.sp.fdy0 : fdy_j[q];
    // output classification (component extents, faces, V0 sets): uy has its
    // y faces at 0 and ny-2, uz at y = 0 and z = N (nz-2), ux at y = 0 (the
    // x = N plane is checked per plane); face points are the face pass's
    own_y[q] = active && !(j == 0 || j == ny - 2);
    own_z[q] = active && !(j == 0 || k == nz - 2);
    own_x[q] = active && j != 0;
  }
  // The z = N face point above an (i, j) that is on no x / y face is one face
  // formula applied to the value this thread computes at k = kz - 1
  // (base_solver.py:552-554, applied last); the thread writes it.  Points on
  // x / y faces as well are left to the face pass.
  const bool zface_xy = k == nz - 2;  // ux, uy: z = N at k = nz-1 (ux: and not the x = N plane)
  const bool zface_z = k == nz - 3;   // uz: z = N at k = nz-2
  const bool rigid = a.bc == 1;

  // -------- TMA ring --------
  // pointwise state is read for the planes whose points this block updates
  const int pw_buf = (S::kahan ? r.rcur : r.rold) * 3;
  auto issue = [&](int p) {  // plane p into its ring slot (one thread)
    const int q = p - ibase, sl = q & (NSLOT - 1);
    const bool pw = p >= ib && p < ie;
    mbar_expect_tx(&bars[sl], P::tx_bytes + (pw ? P::pw_bytes : 0u));
    // test hook (skip_plane >= 0; -1 is off, and plane -1 is a real padding
    // plane that segment 0 loads): armed, no copy, so the wait on it runs out
    if (a.skip_plane >= 0 && p == a.skip_plane) return;
    // padded coordinates: k + KOFF, j + 1, i + 1; the u tiles start at k0-KB, j0-1
    tma_load_4d(uring + sl * SU, &maps->tm_u, k0 - KB + Lay<R>::KOFF, j0, p + 1, r.rcur * 3, &bars[sl]);
    tma_load_3d(mring + sl * SM, &maps->tm_mat, k0, j0, p + 1, &bars[sl]);
    if (pw) {
      R* d = pwring + sl * P::PWS;
      tma_load_4d(d, &maps->tm_pw0, k0 + Lay<R>::KOFF, j0 + 1, p + 1, pw_buf, &bars[sl]);
      if constexpr (S::kahan) tma_load_4d(d + 3 * P::PWC, &maps->tm_pw1, k0 + Lay<R>::KOFF, j0 + 1, p + 1, pw_buf, &bars[sl]);
    }
  };
  bool ok = true;
  auto wait_plane = [&](int p) {
    const int q = p - ibase;
    if (!mbar_wait(&bars[q & (NSLOT - 1)], (q >> 2) & 1, a.wait_polls)) ok = false;
  };
  auto uslot = [&](int p) { return uring + ((p - ibase) & (NSLOT - 1)) * SU; };
  auto mslot = [&](int p) { return mring + ((p - ibase) & (NSLOT - 1)) * SM; };

  if (tid == 0) {
    for (int q = 0; q < NSLOT; q++) mbar_init(&bars[q], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  int issued = ibase - 1;  // last plane issued (thread 0)
  if (tid == 0)
    for (int p = ibase; p <= min(ibase + NSLOT - 1, plast); p++) {
      issue(p);
      issued = p;
    }

  // prologue: planes ib-1 and ib; source patch (plane 0 is in the ring when
  // it is plane ib or ib-1)
  wait_plane(ib - 1);
  wait_plane(ib);
  if (ib <= 1) {
    R* zt = uslot(0) + ZO;
    if (a.source_mode == 1) {
      for (int q = tid; q < CW; q += NT) zt[q] = s;
    } else if (k0 == 0) {
      for (int q = tid; q < TJ + 2; q += NT) zt[q * KW + KB] = s;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();

  // Halo stresses the neighbours need: T2 row j0+TJ, T6 / T4 row j0-1, T3
  // column k0+TK, T4 / T5 column k0-1, one per thread (the first three warps
  // take one row kind each, the next the columns).  All but the plane index
  // is fixed for the tile, so the kind, the smem indices (absolute, tile
  // origin at KW+KB / MKW+MKOFF), the range test and the spacings (with the
  // z = 0 row's substitutions, base_solver.py:420-433) are set up once here.
  static_assert(3 * TK + 3 * TJ <= NT, "one halo task per thread");
  int hk = -1, h_u = 0, h_m = 0, h_dst = 0, h_which = 1;
  bool h_ok = false, h_z0 = false;
  R h_a = R(1), h_b = R(1);
  {
    const int u0 = KW + KB, m0 = MKW + MKOFF;  // tile origin (jl = 0, kl = 0)
    const int qq = tid;
    if (qq < TK) {  // T2 at (j0+TJ, k0+qq)
      const int jj = j0 + TJ, kk = k0 + qq;
      hk = 0;
      h_which = 1;
      h_u = u0 + TJ * KW + qq;
      h_m = m0 + TJ * MKW + qq;
      h_dst = (TJ + 1) * W + qq + 1;
      h_ok = jj >= 1 && jj <= ny - 2 && kk <= nz - 2;
      h_z0 = kk == 0;
      if (h_ok) {
        h_a = h_z0 ? a.sp.sdy0 : __ldg(a.sp.sdy + jj - 1);
        h_b = h_z0 ? a.sp.sdz0 : __ldg(a.sp.sdz + kk - 1);
      }
    } else if (qq < 2 * TK) {  // T6 at (j0-1, k0+q)
      const int q = qq - TK, jj = j0 - 1, kk = k0 + q;
      hk = 1;
      h_u = u0 - KW + q;
      h_m = m0 - MKW + q + MKW;
      h_dst = q + 1;
      h_ok = jj >= 0 && jj <= ny - 2 && kk <= nz - 2;
      h_z0 = kk == 0;
      if (h_ok) h_a = h_z0 ? a.sp.fdx0 : __ldg(a.sp.fdy + jj);
    } else if (qq < 3 * TK) {  // T4 at (j0-1, k0+q)
      const int q = qq - 2 * TK, jj = j0 - 1, kk = k0 + q;
      hk = 2;
      h_u = u0 - KW + q;
      h_m = m0 - MKW + q + MKW + (kk == 0 ? 0 : 1);
      h_dst = q + 1;
      h_ok = jj >= 0 && jj <= ny - 2 && kk <= nz - 2;
      if (h_ok) {
        h_a = kk == 0 ? a.sp.fdy0 : __ldg(a.sp.fdz + kk);
        h_b = kk == 0 ? a.sp.fdz0 : __ldg(a.sp.fdy + jj);
      }
    } else if (qq < 3 * TK + 3 * TJ) {
      const int w = qq - 3 * TK;
      const int which = w / TJ, jl = w - which * TJ;
      const int jj = j0 + jl;
      if (which == 0) {  // T3 at (j0+jl, k0+TK): kk >= 32, never the z = 0 row
        const int kk = k0 + TK;
        hk = 0;
        h_which = 2;
        h_u = u0 + jl * KW + TK;
        h_m = m0 + jl * MKW + TK;
        h_dst = (jl + 1) * W + TK + 1;
        h_ok = jj >= 1 && jj <= ny - 2 && kk <= nz - 2;
        if (h_ok) {
          h_a = __ldg(a.sp.sdy + jj - 1);
          h_b = __ldg(a.sp.sdz + kk - 1);
        }
      } else if (which == 1) {  // T4 at (j0+jl, k0-1): kk >= 31 when valid
        const int kk = k0 - 1;
        hk = 2;
        h_u = u0 + jl * KW - 1;
        h_m = m0 + jl * MKW - 1 + MKW + 1;
        h_dst = (jl + 1) * W;
        h_ok = jj <= ny - 2 && kk >= 0 && kk <= nz - 2;
        if (h_ok) {
          h_a = __ldg(a.sp.fdz + kk);
          h_b = __ldg(a.sp.fdy + jj);
        }
      } else {  // T5 at (j0+jl, k0-1)
        const int kk = k0 - 1;
        hk = 3;
        h_u = u0 + jl * KW - 1;
        h_m = m0 + jl * MKW - 1 + 1;
        h_dst = (jl + 1) * W;
        h_ok = jj >= 1 && jj <= ny - 2 && kk >= 0 && kk <= nz - 2;
        if (h_ok) h_a = __ldg(a.sp.fdz + kk);
      }
    }
  }

  // Values carried from plane to plane instead of re-read from the ring: the
  // stresses of plane i-1 (x differences), ux at i-1 (T1's x difference,
  // ux's own value one plane behind), uy and uz at i (read as plane i+1
  // values one iteration earlier), the material ids of plane i the previous
  // plane's loads fetched.  Prologue: T5, T6 of plane ib-1 and the ring
  // values of planes ib-1, ib.
  R t1m[JR], t5m[JR], t6m[JR], uxm[JR], uxm_up[JR], uyc_n[JR], uzc_n[JR];
  int id_c[JR], id_z[JR], id_y[JR];
  {
    const int i = ib - 1;
    const bool i_s = i >= 0 && i <= nx - 2;
    const R fx = i_s ? __ldg(a.sp.fdx + i) : R(1);
    const R* U0 = uslot(i);
    const R* Up = uslot(i + 1);
    const uint8_t* Mp = mslot(i + 1);
    #pragma unroll
    for (int q = 0; q < JR; q++) {
      const int lu = Lu + q * KW, lm = Lm + q * MKW;
      t5m[q] = R(0);
      t6m[q] = R(0);
      if (i_s && j_n[q] && k_in) {  // T5 (base_solver.py:360-365, 425-428)
        const R c = tab[16 * Mp[lm + (kz ? 0 : 1)] + 10];
        t5m[q] = S::ts(a.dtab, c, S::sub(U0[XO + lu + 1], U0[XO + lu]), kz ? a.sp.fdx0 : fdz_k,
                       S::sub(Up[ZO + lu], U0[ZO + lu]), kz ? a.sp.fdz0 : fx);
      }
      if (i_s && j_s[q] && k_in) {  // T6 (base_solver.py:367-372, 430-433)
        const R c = tab[16 * Mp[lm + MKW] + 11];
        t6m[q] = S::ts(a.dtab, c, S::sub(U0[XO + lu + KW], U0[XO + lu]), kz ? a.sp.fdx0 : fdy_j[q],
                       S::sub(Up[YO + lu], U0[YO + lu]), kz ? a.sp.fdz0 : fx);
      }
      t1m[q] = R(0);
      uxm_up[q] = R(0);
      uxm[q] = U0[XO + lu];
      uyc_n[q] = Up[YO + lu];
      uzc_n[q] = Up[ZO + lu];
      id_c[q] = Mp[lm];
      id_z[q] = Mp[lm + 1];
      id_y[q] = Mp[lm + MKW];
    }
  }

  // the surface record this step writes (none: nullptr), at the own column of row jb
  R* rec = nullptr;
  if (kz && a.record_every > 0 && (tt + 1) % a.record_every == 0) {
    const int slot = (tt + 1) / a.record_every - 1 - a.rec_base;
    if (slot >= 0 && slot < a.nrec_cap) rec = a.surf + ((long long)slot * nx) * ny + jb;
  }

  // element offsets inside one array fit in 32 bits (checked at handle creation)
  const unsigned off_j = (unsigned)(g.o0 + (long long)jb * g.sy + k);  // row r: + r*sy
  const unsigned sxu = (unsigned)g.sx, syu = (unsigned)g.sy;

  // x spacings of plane p: fdx[p] (T5, T6 at p; ux at p+1) and sdx[p-1]
  // (T1..T3 at p; uy, uz at p), read one plane ahead so that their latency
  // is not on the path of the stress evaluation
  // (the spacing arrays are padded: p runs over -1..nx)
  auto fx_at = [&](int p) { return __ldg(a.sp.fdx + p); };
  auto sx_at = [&](int p) { return __ldg(a.sp.sdx + p - 1); };
  R fx_prev = fx_at(ib - 1), fx_cur = fx_at(ib), sx_cur = sx_at(ib);

  for (int i = ib; i <= ie; i++) {
    const unsigned off_i = off_j + (unsigned)i * sxu;  // (i, jb, k)
    const R fx_next = fx_at(i + 1), sx_next = sx_at(i + 1);
    // per-plane (uniform) predicates and spacings
    const bool i_n = i >= 1 && i <= nx - 2;  // T1..T4
    const bool i_s = i <= nx - 2;            // T5, T6 (i >= 0 here)
    const R fdx_i = fx_cur, sdx_im = sx_cur, fdx_im = fx_prev;
    // T1..T3 x spacing, also uy's and uz's x divergence (z = 0 row: sdx[0]);
    // T5, T6 x spacing (z = 0 row: fdz[0]); selected where used
#define SA (kz ? a.sp.sdx0 : sdx_im)
#define SX5 (kz ? a.sp.fdz0 : fdx_i)
    wait_plane(i + 1);
    if (__syncthreads_or(!ok)) break;
    const int p = i & 1;
    const R* Um = uslot(i - 1);
    const R* U0 = uslot(i);
    const R* Up = uslot(i + 1);
    const uint8_t* M0 = mslot(i);
    const uint8_t* Mp = mslot(i + 1);
    // own stresses of plane i, row by row, each ring value read once
    R uxc[JR], uyc[JR], uzc[JR], uxc_up[JR], t1c[JR], t2c[JR], t3c[JR], t4c[JR], t5c[JR], t6c[JR];
    int idp_c[JR], idp_z[JR], idp_y[JR];
    #pragma unroll
    for (int q = 0; q < JR; q++) {
      const int lu = Lu + q * KW, lm = Lm + q * MKW;
      uxc[q] = U0[XO + lu];
      uyc[q] = uyc_n[q];
      uzc[q] = uzc_n[q];
      uyc_n[q] = Up[YO + lu];
      uzc_n[q] = Up[ZO + lu];
      uxc_up[q] = U0[XO + lu + 1];  // ux(i, j, k+1): T5, and the z = N face input of the next plane's ux
      idp_c[q] = Mp[lm];
      idp_z[q] = Mp[lm + 1];
      idp_y[q] = Mp[lm + MKW];
      t1c[q] = t2c[q] = t3c[q] = R(0);
      if (i_n && j_n[q] && k_in) {
        // T1..T3 (base_solver.py:329-351, 408-418): material of the own node
        const R* row = tab + 16 * id_c[q];
        R cc[9];
        if constexpr (sizeof(R) == 4) {
          const float4 q0 = *reinterpret_cast<const float4*>(row), q1 = *reinterpret_cast<const float4*>(row + 4);
          cc[0] = q0.x, cc[1] = q0.y, cc[2] = q0.z, cc[3] = q0.w, cc[4] = q1.x, cc[5] = q1.y, cc[6] = q1.z,
          cc[7] = q1.w;
          cc[8] = row[8];
        } else {
          for (int c = 0; c < 9; c++) cc[c] = row[c];
        }
        const R d1 = S::sub(uxc[q], uxm[q]);
        const R d2 = S::sub(uyc[q], U0[YO + lu - KW]);
        const R d3 = S::sub(uzc[q], U0[ZO + lu - 1]);
        t1c[q] = S::tn1(a.dtab, cc, d1, d2, d3, SA, sb[q], t123_d);
        t2c[q] = S::tn1(a.dtab, cc + 3, d1, d2, d3, SA, sb[q], t123_d);
        if (!kz) t3c[q] = S::tn1(a.dtab, cc + 6, d1, d2, d3, SA, sb[q], t123_d);  // T3[1:-1,1:-1,0] = 0 (:418)
      }
      t4c[q] = t5c[q] = t6c[q] = R(0);
      if (i_n && j_s[q] && k_in) {  // T4 (base_solver.py:353-358, 420-423)
        const R c = tab[16 * (kz ? id_y[q] : (int)M0[lm + MKW + 1]) + 9];
        const R d1 = S::sub(U0[YO + lu + 1], uyc[q]);
        const R d2 = S::sub(U0[ZO + lu + KW], uzc[q]);
        t4c[q] = S::ts(a.dtab, c, d1, kz ? a.sp.fdy0 : fdz_k, d2, kz ? a.sp.fdz0 : fdy_j[q]);
      }
      if (i_s && j_n[q] && k_in) {  // T5 (base_solver.py:360-365, 425-428)
        const R c = tab[16 * (kz ? idp_c[q] : idp_z[q]) + 10];
        const R d1 = S::sub(uxc_up[q], uxc[q]);
        const R d2 = S::sub(uzc_n[q], uzc[q]);
        t5c[q] = S::ts(a.dtab, c, d1, kz ? a.sp.fdx0 : fdz_k, d2, SX5);
      }
      if (i_s && j_s[q] && k_in) {  // T6 (base_solver.py:367-372, 430-433)
        const R c = tab[16 * idp_y[q] + 11];
        const R d1 = S::sub(U0[XO + lu + KW], uxc[q]);
        const R d2 = S::sub(uyc_n[q], uyc[q]);
        t6c[q] = S::ts(a.dtab, c, d1, kz ? a.sp.fdx0 : fdy_j[q], d2, SX5);
      }
      const int l = L + q * W;
      sT2[l] = t2c[q];
      sT3[l] = t3c[q];
      sT4[l] = t4c[q];
      sT5[p * PL + l] = t5c[q];
      sT6[p * PL + l] = t6c[q];
    }
    // this thread's halo stress of plane i (set up before the loop)
    if (hk >= 0) {
      R v = R(0);
      if (hk == 0) {  // T2 row above / T3 column right: one row of the T1-T3 formula
        if (i_n && h_ok) {
          const R* c = tab + 16 * M0[h_m] + 3 * h_which;
          const R d1 = S::sub(U0[XO + h_u], Um[XO + h_u]);
          const R d2 = S::sub(U0[YO + h_u], U0[YO + h_u - KW]);
          const R d3 = S::sub(U0[ZO + h_u], U0[ZO + h_u - 1]);
          v = S::tn1(a.dtab, c, d1, d2, d3, h_z0 ? a.sp.sdx0 : sdx_im, h_a, h_b);
        }
        (h_which == 1 ? sT2 : sT3)[h_dst] = v;
      } else if (hk == 1) {  // T6 row below
        if (i_s && h_ok) {
          const R c = tab[16 * Mp[h_m] + 11];
          const R d1 = S::sub(U0[XO + h_u + KW], U0[XO + h_u]);
          const R d2 = S::sub(Up[YO + h_u], U0[YO + h_u]);
          v = S::ts(a.dtab, c, d1, h_a, d2, h_z0 ? a.sp.fdz0 : fdx_i);
        }
        sT6[p * PL + h_dst] = v;
      } else if (hk == 2) {  // T4 row below / column left
        if (i_n && h_ok) {
          const R c = tab[16 * M0[h_m] + 9];
          const R d1 = S::sub(U0[YO + h_u + 1], U0[YO + h_u]);
          const R d2 = S::sub(U0[ZO + h_u + KW], U0[ZO + h_u]);
          v = S::ts(a.dtab, c, d1, h_a, d2, h_b);
        }
        sT4[h_dst] = v;
      } else {  // T5 column left
        if (i_s && h_ok) {
          const R c = tab[16 * Mp[h_m] + 10];
          const R d1 = S::sub(U0[XO + h_u + 1], U0[XO + h_u]);
          const R d2 = S::sub(Up[ZO + h_u], U0[ZO + h_u]);
          v = S::ts(a.dtab, c, d1, h_a, d2, h_z0 ? a.sp.fdz0 : fdx_i);
        }
        sT5[p * PL + h_dst] = v;
      }
    }
    // ux is updated one plane behind: its pointwise state is taken from the
    // slot of plane i-1 before that slot is refilled
    const R* PWm = pwring + ((i - 1 - ibase) & (NSLOT - 1)) * P::PWS + Lp;  // pointwise, plane i-1
    Pw<R> pwx[JR];
    #pragma unroll
    for (int q = 0; q < JR; q++) pwx[q] = Pw<R>{PWm[q * TK], S::kahan ? PWm[3 * P::PWC + q * TK] : R(0)};
    // The slot of plane i-1 is refilled by a TMA copy (async proxy) that
    // thread 0 issues after the barrier.  A barrier orders shared-memory
    // accesses of the block's threads only: without this proxy fence a read
    // of the slot issued above may still be pending when the copy lands
    // (seen under heavy HBM traffic from other work on the GPU).
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    // plane i-1 is no longer read: refill its slot with plane i-1+NSLOT
    if (tid == 0 && i - 1 + NSLOT <= plast) {
      issue(i - 1 + NSLOT);
      issued = i - 1 + NSLOT;
    }
    const R* PW0 = pwring + ((i - ibase) & (NSLOT - 1)) * P::PWS + Lp;  // pointwise, plane i
    const bool plane_yz = i < ie;                     // uy, uz of plane i belong to this segment
    const bool plane_x = i > ib && i - 1 != nx - 2;  // ux of plane i-1 (not the x = N face)
    const int pm = p ^ 1;
    #pragma unroll
    for (int q = 0; q < JR; q++) {
      const int l = L + q * W, lu = Lu + q * KW;
      const unsigned off = off_i + (unsigned)q * syu;
      if (plane_yz) {
        // uy_new(i, j, k)   (base_solver.py:449-455, 503-509)
        if (own_y[q]) {
          R val;
          if (i_n) {
            // at k = 0 the T4(k-1) halo entry is 0, so T4 - 0 is the z = 0 row's "T4 - 0"
            const R* row = tab + 16 * id_y[q];
            const R dv = S::div3(a.dtab, S::sub(t6c[q], t6m[q]), SA, S::sub(sT2[l + W], t2c[q]), uy_b[q],
                                 S::sub(t4c[q], sT4[l - 1]), t123_d);
            R vn, cn;
            val = update_value<S>(uyc[q], Pw<R>{PW0[P::PWC + q * TK], S::kahan ? PW0[4 * P::PWC + q * TK] : R(0)},
                                  dv, row[12], a.dt, vn, cn);
            store_point<S>(r, 1, off, val, vn, cn);
          } else {
            val = store_stale<S>(r, 1, off);
          }
          if (zface_xy)  // uy on z = N from its inner neighbour (base_solver.py:553)
            store_point<S>(r, 1, off + 1, rigid ? R(0) : S::abc(a.abc[6], val, U0[YO + lu + 1], uyc[q]), R(0), R(0));
        }
        // uz_new(i, j, k)   (base_solver.py:457-463, 511-516)
        if (own_z[q]) {
          R val;
          if (i_n && j_n[q]) {
            // z = 0 row: density at z index 0 (base_solver.py:513); T3(k) = 0 there,
            // and the reference precedence (:516) adds T3[..,1] with factor 1
            const R* row = tab + 16 * (kz ? id_c[q] : id_z[q]);
            const R dv = S::div3(a.dtab, S::sub(t5c[q], t5m[q]), SA, S::sub(t4c[q], sT4[l - W]), sb[q],
                                 S::sub(sT3[l + 1], t3c[q]), uz_c);
            R vn, cn;
            val = update_value<S>(uzc[q],
                                  Pw<R>{PW0[2 * P::PWC + q * TK], S::kahan ? PW0[5 * P::PWC + q * TK] : R(0)}, dv,
                                  row[12], a.dt, vn, cn);
            store_point<S>(r, 2, off, val, vn, cn);
          } else {
            val = store_stale<S>(r, 2, off);
          }
          if (kz) {  // surface uz (base_solver.py:114-116) and the non-finite guard
            if (rec) rec[(long long)i * ny + q] = val;
            if (!isfinite(val)) atomicOr(a.err, 1);
          }
          if (zface_z)  // uz on z = N from its inner neighbour (base_solver.py:554)
            store_point<S>(r, 2, off + 1, rigid ? R(0) : S::abc(a.abc[7], val, U0[ZO + lu + 1], uzc[q]), R(0), R(0));
        }
      }
      if (plane_x && own_x[q]) {
        // ux_new(i-1, j, k)   (base_solver.py:441-447, 495-501)
        const unsigned offm = off - sxu;
        R val;
        if (j_n[q]) {
          const R* row = tab + 16 * id_c[q];  // P[(i-1)+1, j, k]
          // at k = 0 the T5(k-1) halo entry is 0 (the z = 0 row's "T5 - 0")
          const R dv = S::div3(a.dtab, S::sub(t1c[q], t1m[q]), kz ? a.sp.fdx0 : fdx_im,
                               S::sub(sT6[pm * PL + l], sT6[pm * PL + l - W]), sb[q],
                               S::sub(sT5[pm * PL + l], sT5[pm * PL + l - 1]), t123_d);
          R vn, cn;
          val = update_value<S>(uxm[q], pwx[q], dv, row[12], a.dt, vn, cn);
          store_point<S>(r, 0, offm, val, vn, cn);
        } else {
          val = store_stale<S>(r, 0, offm);
        }
        if (zface_xy)  // ux on z = N from its inner neighbour (base_solver.py:552)
          store_point<S>(r, 0, offm + 1, rigid ? R(0) : S::abc(a.abc[6], val, uxm_up[q], uxm[q]), R(0), R(0));
      }
      t1m[q] = t1c[q];
      t5m[q] = t5c[q];
      t6m[q] = t6c[q];
      uxm[q] = uxc[q];
      uxm_up[q] = uxc_up[q];
      id_c[q] = idp_c[q];
      id_z[q] = idp_z[q];
      id_y[q] = idp_y[q];
    }
    fx_prev = fx_cur;
    fx_cur = fx_next;
    sx_cur = sx_next;
#undef SA
#undef SX5
  }
  if (!ok) {
    // A pipeline wait ran out: flag it and drain the copies this block
    // issued, so that no copy writes into this block's shared memory after
    // it returns.  Planes before issued-NSLOT+1 were consumed; the slots of
    // the last NSLOT issued planes are waited for with the full budget (a
    // copy that was issued completes; its phase may already be done, which
    // returns at once).  A plane armed without a copy (the test hook) has
    // nothing in flight and is not waited for.
    if (tid == 0) {
      atomicOr(a.err, 2);
      for (int p = max(ibase, issued - NSLOT + 1); p <= issued; p++) {
        if (a.skip_plane >= 0 && p == a.skip_plane) continue;
        const int q = p - ibase;
        mbar_wait(&bars[q & (NSLOT - 1)], (q >> 2) & 1);
      }
    }
  }
  // every issued plane has been waited for; the barriers may be set up
  // again by the next tile of a persistent block, whose copies write the
  // ring: order this thread's reads of it first (as before a refill)
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  if (tid == 0)
    for (int q = 0; q < NSLOT; q++) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&bars[q])) : "memory");
  __syncthreads();
  return ok;
}
