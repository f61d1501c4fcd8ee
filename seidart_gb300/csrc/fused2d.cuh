// Tile bodies of the single-pass 2-D steps, shared by the per-model kernels
// (fused2d.cu) and the persistent batched kernel (batch.cu).  A tile is
// 32 x (8*ZB) cells handled by a 32 x 8 thread block; thread (tx, ty) owns
// rows z0 + ty + 8 r, r < ZB.
#pragma once
#include "sfd_solvers.h"

namespace sfd {

// ---------------------------------------------------------------------------
// electromag2

// Hy at (i, k) after the H half-step, from the old state
// (electromagfdtd.f95:249-262).  Valid for i <= NX-2, k <= NZ-2.
__device__ __forceinline__ float em2_h_cell(const Em2Step& a, int i, int k, float& pz, float& px, bool& zs,
                                            bool& xs) {
  const int P = a.P, W = a.W;
  const size_t c = (size_t)k * P + i;
  const float dEx = a.Ex0[c + P] - a.Ex0[c];
  float vz = dEx * a.Z.ik[k];
  zs = in_strip(k, a.NZ, W);
  if (zs) {
    pz = a.Z.b[k] * a.mExz0[(size_t)strip_idx(k, a.NZ, W) * P + i] + a.Z.ad[k] * dEx;
    vz += pz;
  }
  const float dEz = a.Ez0[c + 1] - a.Ez0[c];
  float vx = dEz * a.X.ik[i];
  xs = in_strip(i, a.NX, W);
  if (xs) {
    px = a.X.b[i] * a.mEzx0[(size_t)k * (2 * W) + strip_idx(i, a.NX, W)] + a.X.ad[i] * dEz;
    vx += px;
  }
  return a.Hy0[c] + a.dbH * (vx + vz);
}

template <int ZB>
__device__ __forceinline__ void em2_tile(const Em2Step& a, int t, int bx, int by, int gridx, float (*sH)[33]) {
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  const int tx = threadIdx.x, ty = threadIdx.y;
  if (bx == 0 && by == 0 && t > a.io.ctl->run_start) {
    const float* ch[2] = {a.Ex0, a.Ez0};
    gather_receivers<2>(a.io.rec, a.io.nrec, a.io.traces, t - 1, ch, P, 1, false);
  }
  const int x0 = bx * 32, z0 = by * (8 * ZB);
  const int i = x0 + tx;
  // ---- H half-step on the owned cells
#pragma unroll
  for (int r = 0; r < ZB; ++r) {
    const int k = z0 + ty + 8 * r;
    if (i < NX && k < NZ) {
      const size_t c = (size_t)k * P + i;
      float h;
      if (i <= NX - 2 && k <= NZ - 2) {
        float pz = 0.f, px = 0.f;
        bool zs, xs;
        h = em2_h_cell(a, i, k, pz, px, zs, xs);
        if (zs) a.mExz1[(size_t)strip_idx(k, NZ, W) * P + i] = pz;
        if (xs) a.mEzx1[(size_t)k * (2 * W) + strip_idx(i, NX, W)] = px;
        const bool edge = (i == 0) | (i == NX - 2) | (k == 0) | (k == NZ - 2);  // :314-317
        a.Hy1[c] = edge ? 0.0f : h;
      } else {
        h = a.Hy0[c];
        a.Hy1[c] = h;
        if (in_strip(k, NZ, W)) {
          const size_t m = (size_t)strip_idx(k, NZ, W) * P + i;
          a.mExz1[m] = a.mExz0[m];
        }
        if (in_strip(i, NX, W)) {
          const size_t m = (size_t)k * (2 * W) + strip_idx(i, NX, W);
          a.mEzx1[m] = a.mEzx0[m];
        }
      }
      sH[ty + 8 * r + 1][tx + 1] = h;
    }
  }
  // ---- halo: column x0-1 and row z0-1 (not stored)
  if (tx == 0 && x0 > 0) {
#pragma unroll
    for (int r = 0; r < ZB; ++r) {
      const int k = z0 + ty + 8 * r;
      if (k <= NZ - 2) {
        float pz, px;
        bool zs, xs;
        sH[ty + 8 * r + 1][0] = em2_h_cell(a, x0 - 1, k, pz, px, zs, xs);
      }
    }
  }
  if (ty == 0 && z0 > 0 && i <= NX - 2) {
    float pz, px;
    bool zs, xs;
    sH[0][tx + 1] = em2_h_cell(a, i, z0 - 1, pz, px, zs, xs);
  }
  __syncthreads();
  // ---- E half-step, source, Dirichlet, norm on the owned cells
  float norm = 0.0f;
#pragma unroll
  for (int r = 0; r < ZB; ++r) {
    const int k = z0 + ty + 8 * r;
    if (i < NX && k < NZ) {
      const size_t c = (size_t)k * P + i;
      const int kk = ty + 8 * r + 1, ii = tx + 1;
      float ex = a.Ex0[c], ez = a.Ez0[c];
      if (i <= NX - 2 && k >= 1 && k <= NZ - 2) {  // :273-283
        const float dH = sH[kk][ii] - sH[kk - 1][ii];
        float d = dH * a.Z.ikh[k];
        if (in_strip(k, NZ, W)) {
          const size_t m = (size_t)strip_idx(k, NZ, W) * P + i;
          const float psi = a.Z.bh[k] * a.mHyz0[m] + a.Z.adh[k] * dH;
          a.mHyz[m] = psi;
          d += psi;
        }
        ex = 0.5f * (a.caEx[c] + a.caEx[c - P]) * ex + 0.5f * (a.cbEx[c] + a.cbEx[c - P]) * d;
      }
      if (k <= NZ - 2 && i >= 1 && i <= NX - 2) {  // :285-295
        const float dH = sH[kk][ii] - sH[kk][ii - 1];
        float d = dH * a.X.ikh[i];
        if (in_strip(i, NX, W)) {
          const size_t m = (size_t)k * (2 * W) + strip_idx(i, NX, W);
          const float psi = a.X.bh[i] * a.mHyx0[m] + a.X.adh[i] * dH;
          a.mHyx[m] = psi;
          d += psi;
        }
        ez = 0.5f * (a.caEz[c] + a.caEz[c - 1]) * ez + 0.5f * (a.cbEz[c] + a.cbEz[c - 1]) * d;
      }
      if (i == a.io.si && k == a.io.sk) {  // :300-301
        ex += a.io.src[t];
        ez += a.io.src[a.io.nstep + t];
      }
      if (i == 0 || i == NX - 2 || k == 0 || k == NZ - 1) ex = 0.0f;  // :304-312
      if (i == 0 || i == NX - 1 || k == 0 || k == NZ - 2) ez = 0.0f;
      a.Ex1[c] = ex;
      a.Ez1[c] = ez;
      norm = fmaxf(norm, hypotf(ex, ez));
    }
  }
  block_norm_to_slot(norm, a.io.slots, by * gridx + bx);
}

// ---------------------------------------------------------------------------
// seismic2

struct S2Stress {
  float sxx, szz, sxz;
  float mvxx, mvzx, mvzz, mvxz;
  bool xs, zs;
};

// The three stresses at (i, k) after both stress loops of one step, from the
// old state (seismicfdtd.f95:247-312), with the shared velocity-gradient
// memory variables advanced once per loop that visits the cell.
__device__ __forceinline__ S2Stress seis2_stress_cell(const Seis2Step& a, int i, int k) {
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  const size_t c = (size_t)k * P + i;
  S2Stress o;
  o.sxx = a.sxx0[c];
  o.szz = a.szz0[c];
  o.sxz = a.sxz0[c];
  o.xs = in_strip(i, NX, W);
  o.zs = in_strip(k, NZ, W);
  o.mvxx = o.mvzx = o.mvzz = o.mvxz = 0.f;
  const size_t mx = (size_t)k * (2 * W) + (o.xs ? strip_idx(i, NX, W) : 0);
  const size_t mz = (size_t)(o.zs ? strip_idx(k, NZ, W) : 0) * P + i;
  if (o.xs) { o.mvxx = a.m_vxx0[mx]; o.mvzx = a.m_vzx0[mx]; }
  if (o.zs) { o.mvzz = a.m_vzz0[mz]; o.mvxz = a.m_vxz0[mz]; }
  const bool loop1 = (k >= 1) && (i <= NX - 2);
  const bool loop2 = (k <= NZ - 2) && (i >= 1);
  if (!loop1 && !loop2) return o;
  const float vx0 = a.vx0[c], vz0 = a.vz0[c];
  const float ikx = a.X.ik[i], ikxh = a.X.ikh[i], ikz = a.Z.ik[k], ikzh = a.Z.ikh[k];
  const float c15 = a.c15[c], c35 = a.c35[c];
  if (loop1) {
    const float d_vx_x = a.vx0[c + 1] - vx0;
    const float d_vz_z = vz0 - a.vz0[c - P];
    const float d_vz_x = a.vz0[c + 1] - vz0;
    const float d_vx_z = vx0 - a.vx0[c - P];
    if (o.xs) {
      o.mvxx = a.q3[k] * o.mvxx + a.X.adh[i] * d_vx_x;  // b_x_half(j), :255
      o.mvzx = a.X.b[i] * o.mvzx + a.X.ad[i] * d_vz_x;
    }
    if (o.zs) {
      o.mvzz = a.Z.b[k] * o.mvzz + a.Z.ad[k] * d_vz_z;
      o.mvxz = a.Z.bh[k] * o.mvxz + a.Z.adh[k] * d_vx_z;
    }
    const float dvx_dx = d_vx_x * ikxh + o.mvxx;
    const float dvz_dz = d_vz_z * ikz + o.mvzz;
    const float dvz_dx = d_vz_x * ikx + o.mvzx;
    const float dvx_dz = d_vx_z * ikzh + o.mvxz;
    const float A11 = 0.25f * (a.c11[c + 1] + 2.f * a.c11[c] + a.c11[c - P]);
    const float A13 = 0.25f * (a.c13[c + 1] + 2.f * a.c13[c] + a.c13[c - P]);
    const float A15 = 0.25f * (a.c15[c + 1] + 2.f * c15 + a.c15[c - P]);
    const float A33 = 0.25f * (a.c33[c + 1] + 2.f * a.c33[c] + a.c33[c - P]);
    const float A35 = 0.25f * (a.c35[c + 1] + 2.f * c35 + a.c35[c - P]);
    const float shear = dvz_dx + dvx_dz;
    o.sxx = o.sxx + (A11 * dvx_dx + A13 * dvz_dz + A15 * shear);
    o.szz = o.szz + (A13 * dvx_dx + A33 * dvz_dz + A35 * shear);
  }
  if (loop2) {
    const float d_vx_x = vx0 - a.vx0[c - 1];
    const float d_vz_z = a.vz0[c + P] - vz0;
    const float d_vz_x = vz0 - a.vz0[c - 1];
    const float d_vx_z = a.vx0[c + P] - vx0;
    if (o.xs) {
      o.mvxx = a.X.bh[i] * o.mvxx + a.X.adh[i] * d_vx_x;
      o.mvzx = a.X.b[i] * o.mvzx + a.X.ad[i] * d_vz_x;
    }
    if (o.zs) {
      o.mvzz = a.Z.b[k] * o.mvzz + a.Z.ad[k] * d_vz_z;
      o.mvxz = a.Z.bh[k] * o.mvxz + a.Z.adh[k] * d_vx_z;
    }
    const float dvx_dx = d_vx_x * ikxh + o.mvxx;
    const float dvz_dz = d_vz_z * ikz + o.mvzz;
    const float dvz_dx = d_vz_x * ikx + o.mvzx;
    const float dvx_dz = d_vx_z * ikzh + o.mvxz;
    const float B15 = 0.25f * (a.c15[c + P] + 2.f * c15 + a.c15[c - 1]);
    const float B35 = 0.25f * (a.c35[c + P] + 2.f * c35 + a.c35[c - 1]);
    const float B55 = 0.25f * (a.c55[c + P] + 2.f * a.c55[c] + a.c55[c - 1]);
    o.sxz = o.sxz + (B15 * dvx_dx + B35 * dvz_dz + B55 * (dvz_dx + dvx_dz));
  }
  return o;
}

template <int ZB>
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
  // ---- stress half-step on owned cells (stored) and on the halo ring (shared memory only)
#pragma unroll
  for (int r = 0; r < ZB; ++r) {
    const int k = z0 + ty + 8 * r;
    if (i < NX && k < NZ) {
      const size_t c = (size_t)k * P + i;
      const S2Stress s = seis2_stress_cell(a, i, k);
      a.sxx1[c] = s.sxx;
      a.szz1[c] = s.szz;
      a.sxz1[c] = s.sxz;
      if (s.xs) {
        const size_t m = (size_t)k * (2 * W) + strip_idx(i, NX, W);
        a.m_vxx1[m] = s.mvxx;
        a.m_vzx1[m] = s.mvzx;
      }
      if (s.zs) {
        const size_t m = (size_t)strip_idx(k, NZ, W) * P + i;
        a.m_vzz1[m] = s.mvzz;
        a.m_vxz1[m] = s.mvxz;
      }
      sS[0][ty + 8 * r + 1][tx + 1] = s.sxx;
      sS[1][ty + 8 * r + 1][tx + 1] = s.szz;
      sS[2][ty + 8 * r + 1][tx + 1] = s.sxz;
    }
  }
  auto halo = [&](int hi, int hk, int si, int sk) {
    if (hi >= 0 && hi < NX && hk >= 0 && hk < NZ) {
      const S2Stress s = seis2_stress_cell(a, hi, hk);
      sS[0][sk][si] = s.sxx;
      sS[1][sk][si] = s.szz;
      sS[2][sk][si] = s.sxz;
    }
  };
  if (tx == 0) {
#pragma unroll
    for (int r = 0; r < ZB; ++r) halo(x0 - 1, z0 + ty + 8 * r, 0, ty + 8 * r + 1);
  }
  if (tx == 31) {
#pragma unroll
    for (int r = 0; r < ZB; ++r) halo(x0 + 32, z0 + ty + 8 * r, 33, ty + 8 * r + 1);
  }
  if (ty == 0) halo(i, z0 - 1, tx + 1, 0);
  if (ty == 7) halo(i, z0 + 8 * ZB, tx + 1, 8 * ZB + 1);
  __syncthreads();
  // ---- velocity half-step on owned cells (seismicfdtd.f95:317-379)
  float norm = 0.0f;
#pragma unroll
  for (int r = 0; r < ZB; ++r) {
    const int k = z0 + ty + 8 * r;
    if (i < NX && k < NZ) {
      const size_t c = (size_t)k * P + i;
      const int kk = ty + 8 * r + 1, ii = tx + 1;
      const bool xs = in_strip(i, NX, W), zs = in_strip(k, NZ, W);
      const size_t mx = (size_t)k * (2 * W) + (xs ? strip_idx(i, NX, W) : 0);
      const size_t mz = (size_t)(zs ? strip_idx(k, NZ, W) : 0) * P + i;
      const bool interior = (i >= 1) && (i <= NX - 2) && (k >= 1) && (k <= NZ - 2);
      float vx = 0.f, vz = 0.f;
      if (k >= 1 && i >= 1) {  // vx loop, :317-336
        const float d1 = sS[0][kk][ii] - sS[0][kk][ii - 1];
        const float d2 = sS[2][kk][ii] - sS[2][kk - 1][ii];
        float v1 = d1 * a.X.ik[i], v2 = d2 * a.Z.ik[k];
        if (xs) {
          const float m = a.X.b[i] * a.m_sxx_x[mx] + a.X.ad[i] * d1;
          a.m_sxx_x[mx] = m;
          v1 += m;
        }
        if (zs) {
          const float m = a.Z.b[k] * a.m_sxz_z[mz] + a.Z.ad[k] * d2;
          a.m_sxz_z[mz] = m;
          v2 += m;
        }
        if (interior) {
          vx = a.vx0[c];
          if (a.atten) vx *= a.gxp[c];
          vx = vx + (v1 + v2) * a.dtrx[c];
        }
      }
      if (k <= NZ - 2 && i <= NX - 2) {  // vz loop, :338-357
        const float d1 = sS[2][kk][ii + 1] - sS[2][kk][ii];
        const float d2 = sS[1][kk + 1][ii] - sS[1][kk][ii];
        float v1 = d1 * a.X.ikh[i], v2 = d2 * a.Z.ikh[k];
        if (xs) {
          const float m = a.X.bh[i] * a.m_sxz_x[mx] + a.X.adh[i] * d1;
          a.m_sxz_x[mx] = m;
          v1 += m;
        }
        if (zs) {
          const float m = a.Z.bh[k] * a.m_szz_z[mz] + a.Z.adh[k] * d2;
          a.m_szz_z[mz] = m;
          v2 += m;
        }
        if (interior) {
          vz = a.vz0[c];
          if (a.atten) vz *= a.gzp[c];
          vz = vz + (v1 + v2) * a.dtrz[c];
        }
      }
      if (i == a.io.si && k == a.io.sk) {  // :360-361
        vx += a.io.src[t];
        vz += a.io.src[a.io.nstep + t];
      }
      if (!interior) { vx = 0.f; vz = 0.f; }  // :365-375
      a.vx1[c] = vx;
      a.vz1[c] = vz;
      norm = fmaxf(norm, hypotf(vx, vz));
    }
  }
  block_norm_to_slot(norm, a.io.slots, by * gridx + bx);
}

}  // namespace sfd
