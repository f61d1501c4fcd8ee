// Tile bodies of the single-pass 2-D steps, shared by the per-model kernels
// (fused2d.cu) and the persistent batched kernel (batch.cu).  A 32 x 8
// thread block handles a tile of 8*ZB rows: thread (tx, ty) owns rows
// z0 + ty + 8 r, r < ZB, and in each row four consecutive cells (electromag2,
// 128-cell-wide tiles) or one (seismic2, 32-cell-wide tiles).  The one-cell
// halo of the first half-step is
// computed by whole warps (warp w takes one halo side, one cell per lane), so
// no warp diverges lane by lane.  The coefficients and axis tables go
// through the non-coherent cache (__ldg).  So do the fields of the "old"
// copy when the launch writes none of them (RO = true: one launch per step);
// a persistent launch that writes them in its earlier steps (the batched
// kernel) reads them with coherent loads (RO = false).
#pragma once
#include "sfd_solvers.h"

namespace sfd {

template <bool RO>
__device__ __forceinline__ float fld(const float* p) {
  if constexpr (RO) return __ldg(p);
  else return *p;
}
template <bool RO>
__device__ __forceinline__ float4 fld4(const float* p) {
  if constexpr (RO) return __ldg(reinterpret_cast<const float4*>(p));
  else return *reinterpret_cast<const float4*>(p);
}

// ---------------------------------------------------------------------------
// electromag2

// Hy at (i, k) after the H half-step, from the old state
// (electromagfdtd.f95:249-262).  Valid for i <= NX-2, k <= NZ-2.
template <bool RO>
__device__ __forceinline__ float em2_h_cell(const Em2Step& a, int i, int k, float& pz, float& px, bool& zs,
                                            bool& xs) {
  const int P = a.P, W = a.W;
  const int c = k * P + i;
  const float dEx = fld<RO>(a.Ex0 + c + P) - fld<RO>(a.Ex0 + c);
  float vz = dEx * __ldg(a.Z.ik + k);
  zs = in_strip(k, a.NZ, W);
  if (zs) {
    pz = __ldg(a.Z.b + k) * fld<RO>(a.mExz0 + strip_idx(k, a.NZ, W) * P + i) + __ldg(a.Z.ad + k) * dEx;
    vz += pz;
  }
  const float dEz = fld<RO>(a.Ez0 + c + 1) - fld<RO>(a.Ez0 + c);
  float vx = dEz * __ldg(a.X.ik + i);
  xs = in_strip(i, a.NX, W);
  if (xs) {
    px = __ldg(a.X.b + i) * fld<RO>(a.mEzx0 + k * (2 * W) + strip_idx(i, a.NX, W)) + __ldg(a.X.ad + i) * dEz;
    vx += px;
  }
  return fld<RO>(a.Hy0 + c) + a.dbH * (vx + vz);
}

__device__ __forceinline__ float4 ld4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float& el(float4& v, int e) { return (&v.x)[e]; }
__device__ __forceinline__ float el(const float4& v, int e) { return (&v.x)[e]; }

// Shared-memory row width of the em2 tile: column 3 holds the x0-1 halo, the
// 128 tile columns start at 4 so every thread's four cells are one 16-byte slot.
constexpr int kEm2Row = 132;

// Four consecutive cells per thread along x: the tile is 128 x (8*ZB) cells
// and every field, coefficient and table access of a row is one 16-byte load
// or store.
template <int ZB, bool RO>
__device__ __forceinline__ void em2_tile(const Em2Step& a, int t, int bx, int by, int gridx,
                                         float (*sH)[kEm2Row]) {
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  const int tx = threadIdx.x, ty = threadIdx.y;
  if (bx == 0 && by == 0 && t > a.io.ctl->run_start) {
    const float* ch[2] = {a.Ex0, a.Ez0};
    gather_receivers<2>(a.io.rec, a.io.nrec, a.io.traces, t - 1, ch, P, 1, false);
  }
  const int x0 = bx * 128, z0 = by * (8 * ZB);
  const int i0 = x0 + 4 * tx;
  const bool active = i0 < NX;
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 ikx4 = zero4, adx4 = zero4, bx4 = zero4, ikxh4 = zero4, adxh4 = zero4, bxh4 = zero4;
  if (active) {
    ikx4 = ld4(a.X.ik + i0); adx4 = ld4(a.X.ad + i0); bx4 = ld4(a.X.b + i0);
    ikxh4 = ld4(a.X.ikh + i0); adxh4 = ld4(a.X.adh + i0); bxh4 = ld4(a.X.bh + i0);
  }
  const int sx = 4 + 4 * tx;  // shared-memory column of element 0

  // One row of the H half-step for this thread's four cells (k <= NZ-2).
  // Writes the new Hy values to hv; when `own`, also stores Hy and the memory
  // variables of the new copy.
  auto h_row = [&](int k, bool own, float4& hv) {
    const int c0 = k * P + i0;
    const float4 hy = active ? fld4<RO>(a.Hy0 + c0) : zero4;
    const float4 ex = active ? fld4<RO>(a.Ex0 + c0) : zero4;
    const float4 exn = active ? fld4<RO>(a.Ex0 + c0 + P) : zero4;
    const float4 ez = active ? fld4<RO>(a.Ez0 + c0) : zero4;
    float ez_next = __shfl_down_sync(0xffffffffu, ez.x, 1);
    if (tx == 31) ez_next = (i0 + 4 < NX) ? fld<RO>(a.Ez0 + c0 + 4) : 0.f;
    const bool zs = in_strip(k, NZ, W);
    const int zrow = (zs ? strip_idx(k, NZ, W) : 0) * P + i0;
    const float4 pz0 = (zs && active) ? fld4<RO>(a.mExz0 + zrow) : zero4;
    const float ikz = __ldg(a.Z.ik + k), adz = __ldg(a.Z.ad + k), bz = __ldg(a.Z.b + k);
    float4 pz1 = pz0, hy1 = hy;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int i = i0 + e;
      if (i <= NX - 2) {
        const float dEx = el(exn, e) - el(ex, e);
        float vz = dEx * ikz;
        if (zs) {
          el(pz1, e) = bz * el(pz0, e) + adz * dEx;
          vz += el(pz1, e);
        }
        const float dEz = (e < 3 ? el(ez, e + 1) : ez_next) - el(ez, e);
        float vx = dEz * el(ikx4, e);
        if (in_strip(i, NX, W)) {
          const int m = k * (2 * W) + strip_idx(i, NX, W);
          const float px = el(bx4, e) * fld<RO>(a.mEzx0 + m) + el(adx4, e) * dEz;
          if (own) a.mEzx1[m] = px;
          vx += px;
        }
        el(hv, e) = el(hy, e) + a.dbH * (vx + vz);
        const bool edge = (i == 0) | (i == NX - 2) | (k == 0) | (k == NZ - 2);  // :314-317
        el(hy1, e) = edge ? 0.0f : el(hv, e);
      } else {
        el(hv, e) = el(hy, e);
        if (own && i < NX && in_strip(i, NX, W)) {
          const int m = k * (2 * W) + strip_idx(i, NX, W);
          a.mEzx1[m] = fld<RO>(a.mEzx0 + m);
        }
      }
    }
    if (own && active) {
      st4(a.Hy1 + c0, hy1);
      if (zs) st4(a.mExz1 + zrow, pz1);
    }
  };

  // Tiles whose owned cells all lie off the CPML strips, off the Dirichlet
  // planes and away from the source take a path without per-cell masks (the
  // same operations the masked path performs on such cells); their halo row
  // and column still take the general code.
  const int lo = W > 1 ? W : 1;
  const bool fast = x0 >= lo && x0 + 127 <= NX - 1 - lo && x0 + 127 <= NX - 3 && z0 >= lo &&
                    z0 + 8 * ZB - 1 <= NZ - 1 - lo && z0 + 8 * ZB - 1 <= NZ - 3 &&
                    !(a.io.si >= x0 && a.io.si < x0 + 128 && a.io.sk >= z0 && a.io.sk < z0 + 8 * ZB);

  // ---- H half-step on the owned rows
  if (fast) {  // every row computed before the first store (the stores would hold back later loads)
    float4 hv[ZB];
#pragma unroll
    for (int r = 0; r < ZB; ++r) {
      const int k = z0 + ty + 8 * r;
      const int c0 = k * P + i0;
      const float4 hy = fld4<RO>(a.Hy0 + c0), ex = fld4<RO>(a.Ex0 + c0), exn = fld4<RO>(a.Ex0 + c0 + P), ez = fld4<RO>(a.Ez0 + c0);
      float ez_next = __shfl_down_sync(0xffffffffu, ez.x, 1);
      if (tx == 31) ez_next = fld<RO>(a.Ez0 + c0 + 4);
      const float ikz = __ldg(a.Z.ik + k);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float dEx = el(exn, e) - el(ex, e);
        const float vz = dEx * ikz;
        const float dEz = (e < 3 ? el(ez, e + 1) : ez_next) - el(ez, e);
        const float vx = dEz * el(ikx4, e);
        el(hv[r], e) = el(hy, e) + a.dbH * (vx + vz);
      }
    }
#pragma unroll
    for (int r = 0; r < ZB; ++r) {
      st4(a.Hy1 + (z0 + ty + 8 * r) * P + i0, hv[r]);
      *reinterpret_cast<float4*>(&sH[ty + 8 * r + 1][sx]) = hv[r];
    }
  } else {
#pragma unroll
  for (int r = 0; r < ZB; ++r) {
    const int k = z0 + ty + 8 * r;  // uniform across the warp
    if (k < NZ) {
      float4 hv = zero4;
      if (k <= NZ - 2) {
        h_row(k, true, hv);
      } else if (active) {  // row NZ-1 lies outside the H loop: carried over
        const int c0 = k * P + i0;
        hv = fld4<RO>(a.Hy0 + c0);
        st4(a.Hy1 + c0, hv);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          if (i < NX && in_strip(i, NX, W)) {
            const int m = k * (2 * W) + strip_idx(i, NX, W);
            a.mEzx1[m] = fld<RO>(a.mEzx0 + m);
          }
        }
        if (in_strip(k, NZ, W)) {
          const int zrow = strip_idx(k, NZ, W) * P + i0;
          st4(a.mExz1 + zrow, fld4<RO>(a.mExz0 + zrow));
        }
      }
      *reinterpret_cast<float4*>(&sH[ty + 8 * r + 1][sx]) = hv;
    }
  }
  }
  // ---- halo (not stored): warp 0 takes row z0-1, warp 1 column x0-1
  if (ty == 0) {
    if (z0 > 0) {
      float4 hv = zero4;
      h_row(z0 - 1, false, hv);
      *reinterpret_cast<float4*>(&sH[0][sx]) = hv;
    }
  } else if (ty == 1) {
    for (int q = tx; q < 8 * ZB; q += 32) {
      const int k = z0 + q;
      if (x0 > 0 && k <= NZ - 2) {
        float pz, px;
        bool zs, xs;
        sH[q + 1][3] = em2_h_cell<RO>(a, x0 - 1, k, pz, px, zs, xs);
      }
    }
  }
  __syncthreads();
  // ---- E half-step, source, Dirichlet, norm on the owned rows
  float norm = 0.0f;
  if (fast) {  // every row computed before the first store (the stores would hold back later loads)
    float4 exr[ZB], ezr[ZB];
#pragma unroll
    for (int r = 0; r < ZB; ++r) {
      const int k = z0 + ty + 8 * r;
      const int c0 = k * P + i0;
      const int kk = ty + 8 * r + 1;
      float4 ex = fld4<RO>(a.Ex0 + c0), ez = fld4<RO>(a.Ez0 + c0);
      const float4 cax = ld4(a.CAx + c0), cbx = ld4(a.CBx + c0), caz = ld4(a.CAz + c0), cbz = ld4(a.CBz + c0);
      const float4 h = *reinterpret_cast<const float4*>(&sH[kk][sx]);
      const float4 hm = *reinterpret_cast<const float4*>(&sH[kk - 1][sx]);
      const float hl = sH[kk][sx - 1];
      const float ikzh = __ldg(a.Z.ikh + k);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float dHz = el(h, e) - el(hm, e);
        const float exv = el(cax, e) * el(ex, e) + el(cbx, e) * (dHz * ikzh);
        const float dHx = el(h, e) - (e == 0 ? hl : el(h, e > 0 ? e - 1 : 0));
        const float ezv = el(caz, e) * el(ez, e) + el(cbz, e) * (dHx * el(ikxh4, e));
        el(ex, e) = exv;
        el(ez, e) = ezv;
        norm = fmaxf(norm, norm_monitor(exv, ezv));
      }
      exr[r] = ex;
      ezr[r] = ez;
    }
#pragma unroll
    for (int r = 0; r < ZB; ++r) {
      const int c0 = (z0 + ty + 8 * r) * P + i0;
      st4(a.Ex1 + c0, exr[r]);
      st4(a.Ez1 + c0, ezr[r]);
    }
  } else {
#pragma unroll
  for (int r = 0; r < ZB; ++r) {
    const int k = z0 + ty + 8 * r;
    if (k < NZ && active) {
      const int c0 = k * P + i0;
      const int kk = ty + 8 * r + 1;
      float4 ex = fld4<RO>(a.Ex0 + c0), ez = fld4<RO>(a.Ez0 + c0);
      const float4 cax = ld4(a.CAx + c0), cbx = ld4(a.CBx + c0), caz = ld4(a.CAz + c0), cbz = ld4(a.CBz + c0);
      const float4 h = *reinterpret_cast<const float4*>(&sH[kk][sx]);
      const float4 hm = *reinterpret_cast<const float4*>(&sH[kk - 1][sx]);
      const float hl = sH[kk][sx - 1];
      const bool zs = in_strip(k, NZ, W);
      const int zrow = (zs ? strip_idx(k, NZ, W) : 0) * P + i0;
      const float4 pc0 = zs ? *reinterpret_cast<const float4*>(a.mHyz0 + zrow) : zero4;
      float4 pc1 = pc0;
      const float ikzh = __ldg(a.Z.ikh + k), adzh = __ldg(a.Z.adh + k), bzh = __ldg(a.Z.bh + k);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        if (i >= NX) break;
        float exv = el(ex, e), ezv = el(ez, e);
        if (i <= NX - 2 && k >= 1 && k <= NZ - 2) {  // :273-283
          const float dH = el(h, e) - el(hm, e);
          float d = dH * ikzh;
          if (zs) {
            el(pc1, e) = bzh * el(pc0, e) + adzh * dH;
            d += el(pc1, e);
          }
          exv = el(cax, e) * exv + el(cbx, e) * d;
        }
        if (k <= NZ - 2 && i >= 1 && i <= NX - 2) {  // :285-295
          const float dH = el(h, e) - (e == 0 ? hl : el(h, e - 1));
          float d = dH * el(ikxh4, e);
          if (in_strip(i, NX, W)) {
            const int m = k * (2 * W) + strip_idx(i, NX, W);
            const float psi = el(bxh4, e) * a.mHyx0[m] + el(adxh4, e) * dH;
            a.mHyx[m] = psi;
            d += psi;
          }
          ezv = el(caz, e) * ezv + el(cbz, e) * d;
        }
        if (i == a.io.si && k == a.io.sk) {  // :300-301
          exv += a.io.src[t];
          ezv += a.io.src[a.io.nstep + t];
        }
        if (i == 0 || i == NX - 2 || k == 0 || k == NZ - 1) exv = 0.0f;  // :304-312
        if (i == 0 || i == NX - 1 || k == 0 || k == NZ - 2) ezv = 0.0f;
        el(ex, e) = exv;
        el(ez, e) = ezv;
        norm = fmaxf(norm, norm_monitor(exv, ezv));
      }
      st4(a.Ex1 + c0, ex);
      st4(a.Ez1 + c0, ez);
      if (zs) st4(a.mHyz + zrow, pc1);
    }
  }
  }
  block_norm_to_slot(norm, a.io.slots, by * gridx + bx);
}

// ---------------------------------------------------------------------------
// seismic2

struct S2Stress {
  float sxx, szz, sxz;
  float mvxx, mvzx, mvzz, mvxz;  // velocity-gradient memory of the first stress loop (legacy: of both)
  float nvxx, nvzx, nvzz, nvxz;  // the sigmaxz loop's own (corrected physics)
  bool xs, zs;
};

// The three stresses at (i, k) after both stress loops of step t, from the
// old state (seismicfdtd.f95:247-312).  Legacy quirks (a.legacy): the
// velocity-gradient memory variables are shared by the two loops and so
// advance once per loop that visits the cell, and loop 1 reads b_x_half at
// the z index (:255, the q3 table).  Corrected physics: the sigmaxz loop has
// its own four memory variables and loop 1 reads b_x_half(i).  A stress
// source is added after both loops at the source cell.
template <bool RO>
__device__ __forceinline__ S2Stress seis2_stress_cell(const Seis2Step& a, int i, int k, int t) {
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  const int c = k * P + i;
  S2Stress o;
  o.sxx = fld<RO>(a.sxx0 + c);
  o.szz = fld<RO>(a.szz0 + c);
  o.sxz = fld<RO>(a.sxz0 + c);
  o.xs = in_strip(i, NX, W);
  o.zs = in_strip(k, NZ, W);
  o.mvxx = o.mvzx = o.mvzz = o.mvxz = 0.f;
  o.nvxx = o.nvzx = o.nvzz = o.nvxz = 0.f;
  const bool own2 = !a.legacy;
  const int mx = k * (2 * W) + (o.xs ? strip_idx(i, NX, W) : 0);
  const int mz = (o.zs ? strip_idx(k, NZ, W) : 0) * P + i;
  if (o.xs) {
    o.mvxx = fld<RO>(a.m_vxx0 + mx);
    o.mvzx = fld<RO>(a.m_vzx0 + mx);
    if (own2) { o.nvxx = fld<RO>(a.m2_vxx0 + mx); o.nvzx = fld<RO>(a.m2_vzx0 + mx); }
  }
  if (o.zs) {
    o.mvzz = fld<RO>(a.m_vzz0 + mz);
    o.mvxz = fld<RO>(a.m_vxz0 + mz);
    if (own2) { o.nvzz = fld<RO>(a.m2_vzz0 + mz); o.nvxz = fld<RO>(a.m2_vxz0 + mz); }
  }
  const bool loop1 = (k >= 1) && (i <= NX - 2);
  const bool loop2 = (k <= NZ - 2) && (i >= 1);
  if (!loop1 && !loop2) return o;
  const float vx0 = fld<RO>(a.vx0 + c), vz0 = fld<RO>(a.vz0 + c);
  const float ikx = __ldg(a.X.ik + i), ikxh = __ldg(a.X.ikh + i);
  const float ikz = __ldg(a.Z.ik + k), ikzh = __ldg(a.Z.ikh + k);
  if (loop1) {
    const float d_vx_x = fld<RO>(a.vx0 + c + 1) - vx0;
    const float d_vz_z = vz0 - fld<RO>(a.vz0 + c - P);
    const float d_vz_x = fld<RO>(a.vz0 + c + 1) - vz0;
    const float d_vx_z = vx0 - fld<RO>(a.vx0 + c - P);
    if (o.xs) {
      const float bq = a.legacy ? __ldg(a.q3 + k) : __ldg(a.X.bh + i);  // b_x_half(j) as :255, or (i)
      o.mvxx = bq * o.mvxx + __ldg(a.X.adh + i) * d_vx_x;
      o.mvzx = __ldg(a.X.b + i) * o.mvzx + __ldg(a.X.ad + i) * d_vz_x;
    }
    if (o.zs) {
      o.mvzz = __ldg(a.Z.b + k) * o.mvzz + __ldg(a.Z.ad + k) * d_vz_z;
      o.mvxz = __ldg(a.Z.bh + k) * o.mvxz + __ldg(a.Z.adh + k) * d_vx_z;
    }
    const float dvx_dx = d_vx_x * ikxh + o.mvxx;
    const float dvz_dz = d_vz_z * ikz + o.mvzz;
    const float dvz_dx = d_vz_x * ikx + o.mvzx;
    const float dvx_dz = d_vx_z * ikzh + o.mvxz;
    const float A11 = __ldg(a.A11 + c), A13 = __ldg(a.A13 + c), A15 = __ldg(a.A15 + c);
    const float A33 = __ldg(a.A33 + c), A35 = __ldg(a.A35 + c);
    const float shear = dvz_dx + dvx_dz;
    o.sxx = o.sxx + (A11 * dvx_dx + A13 * dvz_dz + A15 * shear);
    o.szz = o.szz + (A13 * dvx_dx + A33 * dvz_dz + A35 * shear);
  }
  if (loop2) {
    const float d_vx_x = vx0 - fld<RO>(a.vx0 + c - 1);
    const float d_vz_z = fld<RO>(a.vz0 + c + P) - vz0;
    const float d_vz_x = vz0 - fld<RO>(a.vz0 + c - 1);
    const float d_vx_z = fld<RO>(a.vx0 + c + P) - vx0;
    float mxx = own2 ? o.nvxx : o.mvxx, mzx = own2 ? o.nvzx : o.mvzx;
    float mzz = own2 ? o.nvzz : o.mvzz, mxz = own2 ? o.nvxz : o.mvxz;
    if (o.xs) {
      mxx = __ldg(a.X.bh + i) * mxx + __ldg(a.X.adh + i) * d_vx_x;
      mzx = __ldg(a.X.b + i) * mzx + __ldg(a.X.ad + i) * d_vz_x;
    }
    if (o.zs) {
      mzz = __ldg(a.Z.b + k) * mzz + __ldg(a.Z.ad + k) * d_vz_z;
      mxz = __ldg(a.Z.bh + k) * mxz + __ldg(a.Z.adh + k) * d_vx_z;
    }
    const float dvx_dx = d_vx_x * ikxh + mxx;
    const float dvz_dz = d_vz_z * ikz + mzz;
    const float dvz_dx = d_vz_x * ikx + mzx;
    const float dvx_dz = d_vx_z * ikzh + mxz;
    o.sxz = o.sxz + (__ldg(a.B15 + c) * dvx_dx + __ldg(a.B35 + c) * dvz_dz +
                     __ldg(a.B55 + c) * (dvz_dx + dvx_dz));
    if (own2) { o.nvxx = mxx; o.nvzx = mzx; o.nvzz = mzz; o.nvxz = mxz; }
    else { o.mvxx = mxx; o.mvzx = mzx; o.mvzz = mzz; o.mvxz = mxz; }
  }
  if (a.io.ssrc && i == a.io.si && k == a.io.sk) {  // stress source: sigma_ij += f_ij(t) dt
    o.sxx += __ldg(a.io.ssrc + t);
    o.szz += __ldg(a.io.ssrc + a.io.nstep + t);
    o.sxz += __ldg(a.io.ssrc + 2 * a.io.nstep + t);
  }
  return o;
}

// The three stresses at (i, k) for a cell off the CPML strips, off the
// Dirichlet planes and away from the source: both stress loops without
// memory variables or masks (the operations the general path performs on
// such a cell).
template <bool RO>
__device__ __forceinline__ void seis2_stress_plain(const Seis2Step& a, int i, int k, float& sxx, float& szz,
                                                   float& sxz) {
  const int P = a.P;
  const int c = k * P + i;
  const float ikx = __ldg(a.X.ik + i), ikxh = __ldg(a.X.ikh + i);
  const float ikz = __ldg(a.Z.ik + k), ikzh = __ldg(a.Z.ikh + k);
  const float vx0 = fld<RO>(a.vx0 + c), vz0 = fld<RO>(a.vz0 + c);
  const float vxl = fld<RO>(a.vx0 + c - 1), vxr = fld<RO>(a.vx0 + c + 1);
  const float vxu = fld<RO>(a.vx0 + c - P), vxd = fld<RO>(a.vx0 + c + P);
  const float vzl = fld<RO>(a.vz0 + c - 1), vzr = fld<RO>(a.vz0 + c + 1);
  const float vzu = fld<RO>(a.vz0 + c - P), vzd = fld<RO>(a.vz0 + c + P);
  sxx = fld<RO>(a.sxx0 + c);
  szz = fld<RO>(a.szz0 + c);
  sxz = fld<RO>(a.sxz0 + c);
  {  // :247-283
    const float dvx_dx = (vxr - vx0) * ikxh, dvz_dz = (vz0 - vzu) * ikz;
    const float dvz_dx = (vzr - vz0) * ikx, dvx_dz = (vx0 - vxu) * ikzh;
    const float A11 = __ldg(a.A11 + c), A13 = __ldg(a.A13 + c), A15 = __ldg(a.A15 + c);
    const float A33 = __ldg(a.A33 + c), A35 = __ldg(a.A35 + c);
    const float shear = dvz_dx + dvx_dz;
    sxx = sxx + (A11 * dvx_dx + A13 * dvz_dz + A15 * shear);
    szz = szz + (A13 * dvx_dx + A33 * dvz_dz + A35 * shear);
  }
  {  // :285-312
    const float dvx_dx = (vx0 - vxl) * ikxh, dvz_dz = (vzd - vz0) * ikz;
    const float dvz_dx = (vz0 - vzl) * ikx, dvx_dz = (vxd - vx0) * ikzh;
    sxz = sxz + (__ldg(a.B15 + c) * dvx_dx + __ldg(a.B35 + c) * dvz_dz + __ldg(a.B55 + c) * (dvz_dx + dvx_dz));
  }
}

template <int ZB, bool RO>
__device__ __forceinline__ void seis2_tile(const Seis2Step& a, int t, int bx, int by, int gridx,
                                           float (*sS)[8 * ZB + 2][34]) {
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  const int tx = threadIdx.x, ty = threadIdx.y;
  if (bx == 0 && by == 0 && t > a.io.ctl->run_start) {
    const float* ch[2] = {a.vx0, a.vz0};
    gather_receivers<2>(a.io.rec, a.io.nrec, a.io.traces, t - 1, ch, P, 1, false);
  }
  const int x0 = bx * 32, z0 = by * (8 * ZB);
  const int i = x0 + tx;
  // Tiles whose owned cells all lie off the CPML strips, off the Dirichlet
  // planes and away from the source take a path without per-cell masks (the
  // same operations the masked path performs on such cells); the halo ring
  // still takes the general code.
  const int lo = W > 1 ? W : 1;
  const bool fast = x0 >= lo && x0 + 31 <= NX - 1 - lo && x0 + 31 <= NX - 2 && z0 >= lo &&
                    z0 + 8 * ZB - 1 <= NZ - 1 - lo && z0 + 8 * ZB - 1 <= NZ - 2 &&
                    !(a.io.si >= x0 && a.io.si < x0 + 32 && a.io.sk >= z0 && a.io.sk < z0 + 8 * ZB);
  // ---- stress half-step on owned cells (stored) ...
  if (fast) {  // every row computed before the first store (the stores would hold back later loads)
    float sxx[ZB], szz[ZB], sxz[ZB];
#pragma unroll
    for (int r = 0; r < ZB; ++r) seis2_stress_plain<RO>(a, i, z0 + ty + 8 * r, sxx[r], szz[r], sxz[r]);
#pragma unroll
    for (int r = 0; r < ZB; ++r) {
      const int c = (z0 + ty + 8 * r) * P + i;
      a.sxx1[c] = sxx[r];
      a.szz1[c] = szz[r];
      a.sxz1[c] = sxz[r];
      sS[0][ty + 8 * r + 1][tx + 1] = sxx[r];
      sS[1][ty + 8 * r + 1][tx + 1] = szz[r];
      sS[2][ty + 8 * r + 1][tx + 1] = sxz[r];
    }
  } else {
#pragma unroll
  for (int r = 0; r < ZB; ++r) {
    const int k = z0 + ty + 8 * r;
    if (i < NX && k < NZ) {
      const int c = k * P + i;
      const S2Stress s = seis2_stress_cell<RO>(a, i, k, t);
      a.sxx1[c] = s.sxx;
      a.szz1[c] = s.szz;
      a.sxz1[c] = s.sxz;
      if (s.xs) {
        const int m = k * (2 * W) + strip_idx(i, NX, W);
        a.m_vxx1[m] = s.mvxx;
        a.m_vzx1[m] = s.mvzx;
        if (!a.legacy) { a.m2_vxx1[m] = s.nvxx; a.m2_vzx1[m] = s.nvzx; }
      }
      if (s.zs) {
        const int m = strip_idx(k, NZ, W) * P + i;
        a.m_vzz1[m] = s.mvzz;
        a.m_vxz1[m] = s.mvxz;
        if (!a.legacy) { a.m2_vzz1[m] = s.nvzz; a.m2_vxz1[m] = s.nvxz; }
      }
      sS[0][ty + 8 * r + 1][tx + 1] = s.sxx;
      sS[1][ty + 8 * r + 1][tx + 1] = s.szz;
      sS[2][ty + 8 * r + 1][tx + 1] = s.sxz;
    }
  }
  }
  // ... and on the halo ring (shared memory only): warps 0-3 take the top
  // row, bottom row, left column and right column, one cell per lane.  When
  // the ring too lies off the strips, the planes and the source, it takes
  // the short path of the owned cells: the ring is these warps' fifth row of
  // work, and the general path would make it the longest.
  const bool fast_ring = fast && x0 - 1 >= lo && x0 + 32 <= NX - 1 - lo && x0 + 32 <= NX - 2 && z0 - 1 >= lo &&
                         z0 + 8 * ZB <= NZ - 1 - lo && z0 + 8 * ZB <= NZ - 2 &&
                         !(a.io.si >= x0 - 1 && a.io.si <= x0 + 32 && a.io.sk >= z0 - 1 && a.io.sk <= z0 + 8 * ZB);
  if (ty < 4) {
    for (int q = tx; q < (ty < 2 ? 32 : 8 * ZB); q += 32) {
      int hi, hk, si, sk;
      if (ty == 0) { hi = x0 + q; hk = z0 - 1; si = q + 1; sk = 0; }
      else if (ty == 1) { hi = x0 + q; hk = z0 + 8 * ZB; si = q + 1; sk = 8 * ZB + 1; }
      else if (ty == 2) { hi = x0 - 1; hk = z0 + q; si = 0; sk = q + 1; }
      else { hi = x0 + 32; hk = z0 + q; si = 33; sk = q + 1; }
      if (fast_ring) {
        float sxx, szz, sxz;
        seis2_stress_plain<RO>(a, hi, hk, sxx, szz, sxz);
        sS[0][sk][si] = sxx;
        sS[1][sk][si] = szz;
        sS[2][sk][si] = sxz;
      } else if (hi >= 0 && hi < NX && hk >= 0 && hk < NZ) {
        const S2Stress s = seis2_stress_cell<RO>(a, hi, hk, t);
        sS[0][sk][si] = s.sxx;
        sS[1][sk][si] = s.szz;
        sS[2][sk][si] = s.sxz;
      }
    }
  }
  __syncthreads();
  // ---- velocity half-step on owned cells (seismicfdtd.f95:317-379)
  float norm = 0.0f;
  if (fast) {  // every row computed before the first store (the stores would hold back later loads)
    float vxr[ZB], vzr[ZB];
    const float ikx = __ldg(a.X.ik + i), ikxh = __ldg(a.X.ikh + i);
#pragma unroll
    for (int r = 0; r < ZB; ++r) {
      const int k = z0 + ty + 8 * r;
      const int c = k * P + i;
      const int kk = ty + 8 * r + 1, ii = tx + 1;
      const float v1 = (sS[0][kk][ii] - sS[0][kk][ii - 1]) * ikx, v2 = (sS[2][kk][ii] - sS[2][kk - 1][ii]) * __ldg(a.Z.ik + k);
      const float w1 = (sS[2][kk][ii + 1] - sS[2][kk][ii]) * ikxh, w2 = (sS[1][kk + 1][ii] - sS[1][kk][ii]) * __ldg(a.Z.ikh + k);
      float vx = fld<RO>(a.vx0 + c), vz = fld<RO>(a.vz0 + c);
      if (a.atten) {
        vx *= __ldg(a.gxp + c);
        vz *= __ldg(a.gzp + c);
      }
      vx = vx + (v1 + v2) * __ldg(a.dtrx + c);
      vz = vz + (w1 + w2) * __ldg(a.dtrz + c);
      vxr[r] = vx;
      vzr[r] = vz;
      norm = fmaxf(norm, norm_monitor(vx, vz));
    }
#pragma unroll
    for (int r = 0; r < ZB; ++r) {
      const int c = (z0 + ty + 8 * r) * P + i;
      a.vx1[c] = vxr[r];
      a.vz1[c] = vzr[r];
    }
  } else {
#pragma unroll
  for (int r = 0; r < ZB; ++r) {
    const int k = z0 + ty + 8 * r;
    if (i < NX && k < NZ) {
      const int c = k * P + i;
      const int kk = ty + 8 * r + 1, ii = tx + 1;
      const bool xs = in_strip(i, NX, W), zs = in_strip(k, NZ, W);
      const int mx = k * (2 * W) + (xs ? strip_idx(i, NX, W) : 0);
      const int mz = (zs ? strip_idx(k, NZ, W) : 0) * P + i;
      const bool interior = (i >= 1) && (i <= NX - 2) && (k >= 1) && (k <= NZ - 2);
      float vx = 0.f, vz = 0.f;
      if (k >= 1 && i >= 1) {  // vx loop, :317-336
        const float d1 = sS[0][kk][ii] - sS[0][kk][ii - 1];
        const float d2 = sS[2][kk][ii] - sS[2][kk - 1][ii];
        float v1 = d1 * __ldg(a.X.ik + i), v2 = d2 * __ldg(a.Z.ik + k);
        if (xs) {
          const float m = __ldg(a.X.b + i) * a.m_sxx_x[mx] + __ldg(a.X.ad + i) * d1;
          a.m_sxx_x[mx] = m;
          v1 += m;
        }
        if (zs) {
          const float m = __ldg(a.Z.b + k) * a.m_sxz_z[mz] + __ldg(a.Z.ad + k) * d2;
          a.m_sxz_z[mz] = m;
          v2 += m;
        }
        if (interior) {
          vx = fld<RO>(a.vx0 + c);
          if (a.atten) vx *= __ldg(a.gxp + c);
          vx = vx + (v1 + v2) * __ldg(a.dtrx + c);
        }
      }
      if (k <= NZ - 2 && i <= NX - 2) {  // vz loop, :338-357
        const float d1 = sS[2][kk][ii + 1] - sS[2][kk][ii];
        const float d2 = sS[1][kk + 1][ii] - sS[1][kk][ii];
        float v1 = d1 * __ldg(a.X.ikh + i), v2 = d2 * __ldg(a.Z.ikh + k);
        if (xs) {
          const float m = __ldg(a.X.bh + i) * a.m_sxz_x[mx] + __ldg(a.X.adh + i) * d1;
          a.m_sxz_x[mx] = m;
          v1 += m;
        }
        if (zs) {
          const float m = __ldg(a.Z.bh + k) * a.m_szz_z[mz] + __ldg(a.Z.adh + k) * d2;
          a.m_szz_z[mz] = m;
          v2 += m;
        }
        if (interior) {
          vz = fld<RO>(a.vz0 + c);
          if (a.atten) vz *= __ldg(a.gzp + c);
          vz = vz + (v1 + v2) * __ldg(a.dtrz + c);
        }
      }
      if (i == a.io.si && k == a.io.sk) {  // :360-361
        vx += a.io.src[t];
        vz += a.io.src[a.io.nstep + t];
      }
      if (!interior) { vx = 0.f; vz = 0.f; }  // :365-375
      a.vx1[c] = vx;
      a.vz1[c] = vz;
      norm = fmaxf(norm, norm_monitor(vx, vz));
    }
  }
  }
  block_norm_to_slot(norm, a.io.slots, by * gridx + bx);
}

}  // namespace sfd
