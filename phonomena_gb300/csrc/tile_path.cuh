// Tile path of the fused step kernel (included by fdtd_step.cu).
//
// A block owns a (TJ x 32) tile of the (y, z) plane and marches along x over
// planes [ib, ie).  Planes of u (3 components, 1-node halo), material ids and
// the pointwise state of the own points (u_old, or v and the Kahan terms)
// arrive by TMA in a 4-slot ring.  Every smem access uses offsets fixed per
// thread (own position Lu / Lm, neighbours at constant distance), the range
// predicates of the reference's slices are split into per-thread (j, k) and
// per-plane (i) parts computed once, and the per-axis spacings live in
// registers, so the inner loop is the stencil arithmetic plus shared-memory
// traffic.  The arithmetic goes through the same scheme primitives (tn1, ts,
// div3, div_surf_ref, update_value) as the face path, operation for
// operation.
// Included inside namespace phono, after SmemPlan and the scheme primitives.
#pragma once

template <class S, int TJ>
__device__ __forceinline__ bool tile_block(const StepArgs<typename S::R>& a, unsigned char* base,
                                           const Roles<typename S::R>& r, const typename S::R s, const int tt,
                                           const int tid, const int b, const StepArgs<typename S::R>* maps) {
  using R = typename S::R;
  using P = SmemPlan<S, TJ>;
  using TF = TileShape<R, TJ>;
  constexpr int NT = TK * TJ;
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
  const int j = j0 + ty, k = k0 + tx;
  const bool active = (j < ny - 1) && (k < nz - 1);
  const int L = (ty + 1) * W + tx + 1;    // own entry of the stress planes
  const int Lu = (ty + 1) * KW + tx + KB;  // own entry of a u component tile
  const int Lm = (ty + 1) * MKW + tx + MKOFF;
  const int Lp = ty * TK + tx;             // own entry of a pointwise component tile

  // the whole material table (nmat <= 256 rows) is staged in shared memory
  for (int q = tid; q < a.nmat * 16; q += NT) stab[q] = __ldg(a.tab + q);
  const R* tab = stab;

  // -------- per-thread constants (own position) --------
  // stress ranges of the reference (base_solver.py:329-372, 408-433)
  const bool k_in = k <= nz - 2;               // all six stresses need k <= nz-2
  const bool j_n = j >= 1 && j <= ny - 2;      // T1..T3, T5: j in [1, ny-2]
  const bool j_s = j <= ny - 2;                // T4, T6: j in [0, ny-2]
  const bool kz = k == 0;                      // traction-free row
  const R sdy_m = j >= 1 && j <= ny - 2 ? __ldg(a.sp.sdy + j - 1) : R(1);
  const R fdy_j = j <= ny - 2 ? __ldg(a.sp.fdy + j) : R(1);
  const R sdz_m = k >= 1 && k <= nz - 2 ? __ldg(a.sp.sdz + k - 1) : R(1);
  const R fdz_k = k <= nz - 2 ? __ldg(a.sp.fdz + k) : R(1);
  // spacings as used by the z = 0 row or the interior (the x ones are per plane)
  const R t123_b = kz ? a.sp.sdy0 : sdy_m, t123_d = kz ? a.sp.sdz0 : sdz_m;
  const R uy_b = kz ? a.sp.fdy0 : fdy_j, uy_c = kz ? a.sp.sdz0 : sdz_m;
  const R uz_b = kz ? a.sp.sdy0 : sdy_m, uz_c = kz ? (a.surface_mode == 0 ? R(1) : a.sp.fdz0) : fdz_k;
  const R ux_b = kz ? a.sp.sdy0 : sdy_m, ux_c = kz ? a.sp.sdz0 : sdz_m;
  // output classification (component extents, faces, V0 sets)
  const bool face_y = j == 0 || j == ny - 2;  // uy: y = 0 / y = N faces
  const bool face_z = j == 0 || k == nz - 2;  // uz: y = 0 / z = N faces
  const bool face_x = j == 0;                 // ux: y = 0 face (x = N checked per plane)
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

  // -------- stress evaluators on plane pointers --------
  // U0/Up: u tiles of planes i and i+1 (Um: i-1); M0/Mp material tiles of i, i+1.
  // d = offset of the evaluated position from the own one inside a tile.
  // The traction-free row (k = 0) differs from the interior only in the
  // spacings and material index it uses: its "uz - 0" is the interior
  // difference against the zero padding at k = -1.  So each stress is one
  // evaluation on selected operands, never two evaluations and a select.
  // T5 (base_solver.py:360-365, 425-428)
  auto T5f = [&](const R* U0, const R* Up, const uint8_t* Mp, int du, int dm, bool kzero, R fz, R fx) {
    const R c = tab[16 * Mp[Lm + dm + (kzero ? 0 : 1)] + 10];
    const R d1 = S::sub(U0[XO + Lu + du + 1], U0[XO + Lu + du]);
    const R d2 = S::sub(Up[ZO + Lu + du], U0[ZO + Lu + du]);
    return S::ts(a.dtab, c, d1, kzero ? a.sp.fdx0 : fz, d2, kzero ? a.sp.fdz0 : fx);
  };
  // T6 (base_solver.py:367-372, 430-433)
  auto T6f = [&](const R* U0, const R* Up, const uint8_t* Mp, int du, int dm, bool kzero, R fy, R fx) {
    const R c = tab[16 * Mp[Lm + dm + MKW] + 11];
    const R d1 = S::sub(U0[XO + Lu + du + KW], U0[XO + Lu + du]);
    const R d2 = S::sub(Up[YO + Lu + du], U0[YO + Lu + du]);
    return S::ts(a.dtab, c, d1, kzero ? a.sp.fdx0 : fy, d2, kzero ? a.sp.fdz0 : fx);
  };

  // Halo stresses the neighbours need: T2 row j0+TJ, T6 / T4 row j0-1, T3
  // column k0+TK, T4 / T5 column k0-1, one per thread (the first three warps
  // take one row kind each, the next the columns; 3*TK + 3*TJ <= TK*TJ).
  // All but the plane index is fixed for the tile, so the kind, the smem
  // indices (absolute, tile origin at KW+KB / MKW+MKOFF), the range test and
  // the spacings (with the z = 0 row's substitutions, base_solver.py:420-433)
  // are set up once here.
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

  // prologue stresses: own T5, T6 at plane ib-1
  R t5m, t6m;
  {
    const int i = ib - 1;
    const bool i_s = i >= 0 && i <= nx - 2;
    const R fx = i_s ? __ldg(a.sp.fdx + i) : R(1);
    const R* U0 = uslot(i);
    const R* Up = uslot(i + 1);
    const uint8_t* Mp = mslot(i + 1);
    t5m = (i_s && j_n && k_in) ? T5f(U0, Up, Mp, 0, 0, kz, fdz_k, fx) : R(0);
    t6m = (i_s && j_s && k_in) ? T6f(U0, Up, Mp, 0, 0, kz, fdy_j, fx) : R(0);
  }
  R t1m = 0, uxm_up = 0;
  // values carried from plane to plane instead of re-read from the ring:
  // ux at i-1 (T1's x difference, ux's own value one plane behind), uy and
  // uz at i (read as plane i+1 values one iteration earlier), and the
  // material ids of plane i the next plane's loads already fetched
  R uxm = uslot(ib - 1)[XO + Lu];
  R uyc_n = uslot(ib)[YO + Lu], uzc_n = uslot(ib)[ZO + Lu];
  int id_c = mslot(ib)[Lm], id_z = mslot(ib)[Lm + 1], id_y = mslot(ib)[Lm + MKW];

  // which component updates this thread owns (loop-invariant), and the
  // surface record this step writes (none: nullptr)
  const bool own_y = active && !face_y, own_z = active && !face_z, own_x = active && !face_x;
  R* rec = nullptr;
  if (kz && a.record_every > 0 && (tt + 1) % a.record_every == 0) {
    const int slot = (tt + 1) / a.record_every - 1 - a.rec_base;
    if (slot >= 0 && slot < a.nrec_cap) rec = a.surf + ((long long)slot * nx) * ny + j;
  }

  // element offsets inside one array fit in 32 bits (checked at handle creation)
  const unsigned off_j = (unsigned)(g.o0 + (long long)j * g.sy + k);
  const unsigned sxu = (unsigned)g.sx;

  // x spacings of plane p: fdx[p] (T5, T6 at p; ux at p+1) and sdx[p-1]
  // (T1..T3 at p; uy, uz at p), read one plane ahead so that their latency
  // is not on the path of the stress evaluation
  // (the spacing arrays are padded: p runs over -1..nx)
  auto fx_at = [&](int p) { return __ldg(a.sp.fdx + p); };
  auto sx_at = [&](int p) { return __ldg(a.sp.sdx + p - 1); };
  R fx_prev = fx_at(ib - 1), fx_cur = fx_at(ib), sx_cur = sx_at(ib);

  for (int i = ib; i <= ie; i++) {
    const unsigned off_i = off_j + (unsigned)i * sxu;  // (i, j, k)
    const R fx_next = fx_at(i + 1), sx_next = sx_at(i + 1);
    // per-plane (uniform) predicates and spacings
    const bool i_n = i >= 1 && i <= nx - 2;  // T1..T4
    const bool i_s = i <= nx - 2;            // T5, T6 (i >= 0 here)
    const R fdx_i = fx_cur, sdx_im = sx_cur, fdx_im = fx_prev;
    wait_plane(i + 1);
    if (__syncthreads_or(!ok)) break;
    const int p = i & 1;
    const R* Um = uslot(i - 1);
    const R* U0 = uslot(i);
    const R* Up = uslot(i + 1);
    const uint8_t* M0 = mslot(i);
    const uint8_t* Mp = mslot(i + 1);
    // own stresses at plane i, each read of the ring once
    const R uxc = U0[XO + Lu], uyc = uyc_n, uzc = uzc_n;
    uyc_n = Up[YO + Lu];
    uzc_n = Up[ZO + Lu];
    const R uxc_up = U0[XO + Lu + 1];  // ux(i, j, k+1): T5, and the z = N face input of the next plane's ux
    const int idp_c = Mp[Lm], idp_z = Mp[Lm + 1], idp_y = Mp[Lm + MKW];
    R t1c = R(0), t2c = R(0), t3c = R(0);
    if (i_n && j_n && k_in) {
      // T1..T3 (base_solver.py:329-351, 408-418): material of the own node
      const R* row = tab + 16 * id_c;
      R cc[9];
      if constexpr (sizeof(R) == 4) {
        const float4 q0 = *reinterpret_cast<const float4*>(row), q1 = *reinterpret_cast<const float4*>(row + 4);
        cc[0] = q0.x, cc[1] = q0.y, cc[2] = q0.z, cc[3] = q0.w, cc[4] = q1.x, cc[5] = q1.y, cc[6] = q1.z, cc[7] = q1.w;
        cc[8] = row[8];
      } else {
        for (int q = 0; q < 9; q++) cc[q] = row[q];
      }
      const R d1 = S::sub(uxc, uxm);
      const R d2 = S::sub(uyc, U0[YO + Lu - KW]);
      const R d3 = S::sub(uzc, U0[ZO + Lu - 1]);
      const R sa = kz ? a.sp.sdx0 : sdx_im;
      t1c = S::tn1(a.dtab, cc, d1, d2, d3, sa, t123_b, t123_d);
      t2c = S::tn1(a.dtab, cc + 3, d1, d2, d3, sa, t123_b, t123_d);
      if (!kz) t3c = S::tn1(a.dtab, cc + 6, d1, d2, d3, sa, t123_b, t123_d);  // T3[1:-1,1:-1,0] = 0 (:418)
    }
    R t4c = R(0), t5c = R(0), t6c = R(0);
    if (i_n && j_s && k_in) {  // T4 (base_solver.py:353-358, 420-423)
      const R c = tab[16 * (kz ? id_y : (int)M0[Lm + MKW + 1]) + 9];
      const R d1 = S::sub(U0[YO + Lu + 1], uyc);
      const R d2 = S::sub(U0[ZO + Lu + KW], uzc);
      t4c = S::ts(a.dtab, c, d1, kz ? a.sp.fdy0 : fdz_k, d2, kz ? a.sp.fdz0 : fdy_j);
    }
    if (i_s && j_n && k_in) {  // T5 (base_solver.py:360-365, 425-428)
      const R c = tab[16 * (kz ? idp_c : idp_z) + 10];
      const R d1 = S::sub(uxc_up, uxc);
      const R d2 = S::sub(uzc_n, uzc);
      t5c = S::ts(a.dtab, c, d1, kz ? a.sp.fdx0 : fdz_k, d2, kz ? a.sp.fdz0 : fdx_i);
    }
    if (i_s && j_s && k_in) {  // T6 (base_solver.py:367-372, 430-433)
      const R c = tab[16 * idp_y + 11];
      const R d1 = S::sub(U0[XO + Lu + KW], uxc);
      const R d2 = S::sub(uyc_n, uyc);
      t6c = S::ts(a.dtab, c, d1, kz ? a.sp.fdx0 : fdy_j, d2, kz ? a.sp.fdz0 : fdx_i);
    }
    sT2[L] = t2c;
    sT3[L] = t3c;
    sT4[L] = t4c;
    sT5[p * PL + L] = t5c;
    sT6[p * PL + L] = t6c;
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
    const Pw<R> pwx{PWm[0], S::kahan ? PWm[3 * P::PWC] : R(0)};
    __syncthreads();
    // plane i-1 is no longer read: refill its slot with plane i-1+NSLOT
    if (tid == 0 && i - 1 + NSLOT <= plast) {
      issue(i - 1 + NSLOT);
      issued = i - 1 + NSLOT;
    }
    const R* PW0 = pwring + ((i - ibase) & (NSLOT - 1)) * P::PWS + Lp;  // pointwise, plane i
    const bool plane_yz = i < ie;                            // uy, uz of plane i belong to this segment
    const bool plane_x = i > ib && i - 1 != nx - 2;         // ux of plane i-1 (not the x = N face)
    {
      if (plane_yz) {
        // uy_new(i, j, k)   (base_solver.py:449-455, 503-509)
        if (own_y) {
          R val;
          if (i_n) {
            // at k = 0 the T4(k-1) halo entry is 0, so T4 - 0 is the z = 0 row's "T4 - 0"
            const R* row = tab + 16 * id_y;
            const R dv = S::div3(a.dtab, S::sub(t6c, t6m), kz ? a.sp.sdx0 : sdx_im, S::sub(sT2[L + W], t2c), uy_b,
                                 S::sub(t4c, sT4[L - 1]), uy_c);
            R vn, cn;
            val = update_value<S>(uyc, Pw<R>{PW0[P::PWC], S::kahan ? PW0[4 * P::PWC] : R(0)}, dv, row[12], a.dt, vn,
                                  cn);
            store_point<S>(r, 1, off_i, val, vn, cn);
          } else {
            val = store_stale<S>(r, 1, off_i);
          }
          if (zface_xy)  // uy on z = N from its inner neighbour (base_solver.py:553)
            store_point<S>(r, 1, off_i + 1, rigid ? R(0) : S::abc(a.abc[6], val, U0[YO + Lu + 1], uyc), R(0), R(0));
        }
        // uz_new(i, j, k)   (base_solver.py:457-463, 511-516)
        if (own_z) {
          R val;
          if (i_n && j_n) {
            // z = 0 row: density at z index 0 (base_solver.py:513); T3(k) = 0 there,
            // and the reference precedence (:516) adds T3[..,1] with factor 1
            const R* row = tab + 16 * (kz ? id_c : id_z);
            const R dv = S::div3(a.dtab, S::sub(t5c, t5m), kz ? a.sp.sdx0 : sdx_im, S::sub(t4c, sT4[L - W]), uz_b,
                                 S::sub(sT3[L + 1], t3c), uz_c);
            R vn, cn;
            val = update_value<S>(uzc, Pw<R>{PW0[2 * P::PWC], S::kahan ? PW0[5 * P::PWC] : R(0)}, dv, row[12], a.dt,
                                  vn, cn);
            store_point<S>(r, 2, off_i, val, vn, cn);
          } else {
            val = store_stale<S>(r, 2, off_i);
          }
          if (kz) {  // surface uz (base_solver.py:114-116) and the non-finite guard
            if (rec) rec[(long long)i * ny] = val;
            if (!isfinite(val)) atomicOr(a.err, 1);
          }
          if (zface_z)  // uz on z = N from its inner neighbour (base_solver.py:554)
            store_point<S>(r, 2, off_i + 1, rigid ? R(0) : S::abc(a.abc[7], val, U0[ZO + Lu + 1], uzc), R(0), R(0));
        }
      }
      if (plane_x && own_x) {
        // ux_new(i-1, j, k)   (base_solver.py:441-447, 495-501)
        const unsigned off = off_i - sxu;
        R val;
        if (j_n) {
          const int pm = p ^ 1;
          const R* row = tab + 16 * id_c;  // P[(i-1)+1, j, k]
          // at k = 0 the T5(k-1) halo entry is 0 (the z = 0 row's "T5 - 0")
          const R dv = S::div3(a.dtab, S::sub(t1c, t1m), kz ? a.sp.fdx0 : fdx_im,
                               S::sub(sT6[pm * PL + L], sT6[pm * PL + L - W]), ux_b,
                               S::sub(sT5[pm * PL + L], sT5[pm * PL + L - 1]), ux_c);
          R vn, cn;
          val = update_value<S>(uxm, pwx, dv, row[12], a.dt, vn, cn);
          store_point<S>(r, 0, off, val, vn, cn);
        } else {
          val = store_stale<S>(r, 0, off);
        }
        if (zface_xy)  // ux on z = N from its inner neighbour (base_solver.py:552)
          store_point<S>(r, 0, off + 1, rigid ? R(0) : S::abc(a.abc[6], val, uxm_up, uxm), R(0), R(0));
      }
    }
    t1m = t1c;
    t5m = t5c;
    t6m = t6c;
    fx_prev = fx_cur;
    fx_cur = fx_next;
    sx_cur = sx_next;
    uxm = uxc;
    uxm_up = uxc_up;
    id_c = idp_c;
    id_z = idp_z;
    id_y = idp_y;
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
  // again by the next tile of a persistent block
  __syncthreads();
  if (tid == 0)
    for (int q = 0; q < NSLOT; q++) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&bars[q])) : "memory");
  __syncthreads();
  return ok;
}

