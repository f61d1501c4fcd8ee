// On-chip adjoint sweep of the electromag2 step: every transposed step of a
// checkpoint segment in one cooperative launch, with the adjoint state on
// chip.
//
// The transposed step is the one of the per-step adjoint kernels
// (adjoint_em2.cu), i.e. the exact transpose of
// legacy/fortran/electromagfdtd.f95:249-321 in reverse order:
//   receivers:  lam_Ex, lam_Ez += dJ/d(trace) at the receiver cells;
//   phase A (E half transposed), per cell, from the masked lam_E:
//     gx = CBx lam_Ex (ikh_z + adh_z) + lam_C adh_z       (Ex range)
//     gz = CBz lam_Ez (ikh_x + adh_x) + lam_D adh_x       (Ez range)
//     TH(i,k) = lam_Hy + gx(i,k) - gx(i,k+1) + gz(i,k) - gz(i+1,k)
//     lam_Ex <- CAx lam_Ex, lam_Ez <- CAz lam_Ez, lam_C, lam_D decayed,
//     dJ/dCA += lam_E E, dJ/dCB += lam_E (dH ikh + psi'), source term;
//   phase B (H half transposed), per cell, from TH:
//     hA = dbH TH (ik_z + ad_z) + lam_A ad_z,  hB = dbH TH (ik_x + ad_x) + lam_B ad_x
//     lam_Ex += hA(i,k-1) - hA(i,k), lam_Ez += hB(i-1,k) - hB(i,k),
//     lam_Hy <- TH (zero on its Dirichlet planes), lam_A, lam_B decayed.
// Phase A needs gx of the row below and gz of the column to the right,
// phase B hA of the row above and hB of the column to the left: the same
// directions as the forward H and E halves, so the tiling, the thread
// layout (four cells of kResRows rows per thread, the last warp moving the
// tile's edges) and the tagged edge words of the forward run (resident2d.cu)
// carry over unchanged.  Field 0 of the edge words holds gx / gz (first row,
// first column), field 1 holds hA / hB (last row, last column).
//
// lam_Ex, lam_Ez, lam_Hy of a thread's cells stay in its registers; the
// coefficients, the adjoint memory variables, the gradient sums and the axis
// tables stay in shared memory.  The forward state of each step (Ex, Ez,
// Hy' -- Hy after the H half, before its Dirichlet planes are zeroed -- and
// psi' on the strips) comes from the per-step copies a recompute run
// (resident2d.cu with a ResDump) wrote just before: each thread copies the
// Ex, Ez, Hy' of its cells for the next transposed step into shared memory
// with cp.async while it runs phase B, and prefetches the strips' psi' into
// L2.
#include <algorithm>

#include "resident_common.cuh"

namespace sfd {

using namespace res;

namespace {

// Per-cell masks of a thread, four bits each (bit e = cell 4tx+e).
enum : unsigned {
  kAEX = 0,    // Ex is updated: i <= NX-2, 1 <= k <= NZ-2
  kAEZ = 4,    // Ez is updated: 1 <= i <= NX-2, k <= NZ-2
  kAH = 8,     // Hy is updated: i <= NX-2, k <= NZ-2
  kAXE = 12,   // Ex Dirichlet plane: i == 0, NX-2 or k == 0, NZ-1
  kAZE = 16,   // Ez Dirichlet plane: i == 0, NX-1 or k == 0, NZ-2
  kAHE = 20,   // Hy Dirichlet plane: i == 0, NX-2 or k == 0, NZ-2
  kAXS = 24,   // in the x-strip
  kACELL = 28  // i < NX
};

// Rows of the tile's axis tables in shared memory.
enum { kTKH, kTADH, kTBH, kTIKH, kTK, kTAD, kTB, kNT };

// Array q (0..6: Ex Ez Hy A B C D) of forward slot s.
// 16-byte copy from global to shared memory that completes asynchronously
// (cp.async, through L2); cp_async_wait_all makes the thread's own copies
// visible to it.
__device__ __forceinline__ void cp_async16(float* sdst, const float* gsrc) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(sdst)),
               "l"(gsrc)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

__device__ __forceinline__ const float* slot_f(const Em2AdjResident& a, int s, int q) {
  return (const float*)(a.slots + (size_t)s * a.stride + a.off[q]);
}

// Whether the group of four columns from i holds a cell of the x-strip.
__host__ __device__ inline bool strip_group(int i, int NX, int W) { return i < W || i + 3 >= NX - W; }

// Rows of a tile (columns [x0, x0 + TW), rows [z0, z0 + TZ)) in the z-strip
// and its groups of four columns holding x-strip cells.
__host__ __device__ inline void adj_tile_strips(int x0, int TW, int z0, int TZ, int NX, int NZ, int W, int* nzr,
                                                int* nxg) {
  auto imax = [](int u, int v) { return u > v ? u : v; };
  auto imin = [](int u, int v) { return u < v ? u : v; };
  const int z1 = z0 + TZ, zbot = imax(z0, imax(W, NZ - W));
  *nzr = imax(0, imin(W, z1) - z0) + imax(0, z1 - zbot);
  int n = 0;
  for (int q = 0; 4 * q < TW; ++q) n += strip_group(x0 + 4 * q, NX, W) ? 1 : 0;
  *nxg = n;
}

__device__ __forceinline__ bool hy_plane(int i, int k, int NX, int NZ) {
  return i == 0 || i == NX - 2 || k == 0 || k == NZ - 2;
}

__device__ __forceinline__ void prefetch_l2(const float* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

__global__ void __launch_bounds__(kResThreads, 1) em2_adj_resident_kernel(const __grid_constant__ Em2AdjResident a) {
  constexpr int RB = kResRows;
  extern __shared__ __align__(16) float smem[];
  __shared__ int s_abort, s_nrec;
  __shared__ int s_rec[2 * kResMaxLocalRec];  // (receiver, tile cell) pairs
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  const int4 te = a.plan.tile[blockIdx.x];
  const int x0 = te.x & 0xffff, z0 = te.y & 0xffff, bz = te.z & 0xffff, bx = te.z >> 16;
  const int nxt = (te.x >> 16) - x0, nzt = (te.y >> 16) - z0;
  const int TW = (nxt + 3) & ~3, TZ = nzt;
  const int TXT = TW >> 2, TYT = (TZ + RB - 1) / RB, SX = TXT + 1;
  const bool up = bz > 0, down = bz < a.plan.ntz - 1, left = bx > 0, right = bx < (te.w & 0xffff) - 1;
  const int tid = threadIdx.x;
  const bool xwarp = tid >= kResCellThreads;
  int cls = 3;
  if (!xwarp && tid < TXT * TYT) {
    const int gi = x0 + 4 * (tid % TXT), gk0 = z0 + RB * (tid / TXT);
    const int gk1 = min(gk0 + RB, z0 + nzt) - 1;
    const bool edge = gi < 1 || gi + 3 > NX - 3 || gk0 < 1 || gk1 > NZ - 3 ||
                      (a.sk >= gk0 && a.sk <= gk1 && a.si >= gi && a.si < gi + 4);
    const bool strp = in_strip(gk0, NZ, W) || in_strip(gk1, NZ, W) || in_strip(gi, NX, W) || in_strip(gi + 3, NX, W);
    cls = edge ? 2 : (strp ? 1 : 0);
  }
  const int g = class_ordered_group<3>(cls);
  const int tx = g >= 0 ? g % TXT : 0, ty = g >= 0 ? g / TXT : 0;
  const int rbase = RB * ty;
  const int nrows = g >= 0 ? min(RB, nzt - rbase) : 0;
  const bool cell = nrows > 0;
  const int i0 = x0 + 4 * tx;
  // float4-accessed arrays first (CS and TW are multiples of 4).  The
  // coefficients and gradient sums are read only by the owning thread and
  // indexed by thread: row j of thread tid is the float4 at
  // so = 4 (j * kResCellThreads + tid), conflict-free whichever groups a
  // warp's threads own.
  const int CS = 4 * RB * kResCellThreads;
  float* sCAx = smem;
  float* sCBx = sCAx + CS;
  float* sCAz = sCBx + CS;
  float* sCBz = sCAz + CS;
  float* sGAx = sCBz + CS;  // gradient sums of the sweep
  float* sGBx = sGAx + CS;
  float* sGAz = sGBx + CS;
  float* sGBz = sGAz + CS;
  // adjoint memory variables of the tile's strip cells only: lam_A, lam_C of
  // its nzr z-strip rows ([nzr][TW]), lam_B, lam_D of its nxg x-strip
  // groups ([TZ][4 nxg])
  int nzr, nxg;
  adj_tile_strips(x0, TW, z0, TZ, NX, NZ, W, &nzr, &nxg);
  const int XS = 4 * nxg;
  // the forward Ex, Ez and Hy' of the thread's cells for the next transposed
  // step, copied in one step ahead (cp.async) and indexed like the above
  float* sSEx = sGBz + CS;
  float* sSEz = sSEx + CS;
  float* sSHy = sSEz + CS;
  float* sLA = sSHy + CS;
  float* sLC = sLA + nzr * TW;
  float* sLB = sLC + nzr * TW;
  float* sLD = sLB + TZ * XS;
  float* sGxRow = sLD + TZ * XS;            // [TYT+1][TW]: gx of the first row of thread row ty; row TYT = tile below
  float* sHaRow = sGxRow + (TYT + 1) * TW;  // [TYT+1][TW]: row ty+1 = hA of the last row of thread row ty; row 0 = tile above
  float* sXt = sHaRow + (TYT + 1) * TW;     // [kNT][TW]
  float* sZt = sXt + kNT * TW;              // [kNT][TZ]
  float* sGzCol = sZt + kNT * TZ;           // [TZ][SX]: gz of the first column of thread column tx; column TXT = tile right
  float* sHbCol = sGzCol + TZ * SX;         // [TZ][SX]: column tx+1 = hB of the last column of tx; column 0 = tile left
  const int nsm = 11 * CS + 2 * nzr * TW + 2 * TZ * XS + 2 * (TYT + 1) * TW + kNT * TW + kNT * TZ + 2 * TZ * SX;
  // offsets of a row of this thread's cells in the z-strip and x-strip arrays
  const int zbot = max(z0, max(W, NZ - W)), ntop = max(0, min(W, z0 + TZ) - z0);
  int xgi = 0;  // x-strip groups left of this thread's group
  for (int q = 0; q < tx; ++q) xgi += strip_group(x0 + 4 * q, NX, W) ? 1 : 0;
  auto zoff = [&](int row) { return (z0 + row < W ? row : ntop + z0 + row - zbot) * TW + 4 * tx; };
  auto xoff = [&](int row) { return row * XS + 4 * xgi; };
  const int NZp = a.r.NZp;
  auto erow = [&](int par, int f, int b) { return a.r.erow + (size_t)((par * 2 + f) * kResMaxTiles1D + b) * P; };
  auto ecol = [&](int par, int f, int b) { return a.r.ecol + (size_t)((par * 2 + f) * kResMaxTiles1D + b) * NZp; };
  Ctl* ctl = a.ctl;
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);

  for (int q = tid; q < nsm; q += blockDim.x) smem[q] = 0.0f;
  if (tid == 0) {
    s_nrec = 0;
    s_abort = 0;
  }
  __syncthreads();

  // ---- axis tables of the tile
  for (int c = tid; c < TW; c += blockDim.x) {
    const int i = x0 + c;
    if (i < NX) {
      const float ikh = __ldg(a.X.ikh + i), adh = __ldg(a.X.adh + i), ik = __ldg(a.X.ik + i), ad = __ldg(a.X.ad + i);
      sXt[kTKH * TW + c] = ikh + adh;
      sXt[kTADH * TW + c] = adh;
      sXt[kTBH * TW + c] = __ldg(a.X.bh + i);
      sXt[kTIKH * TW + c] = ikh;
      sXt[kTK * TW + c] = ik + ad;
      sXt[kTAD * TW + c] = ad;
      sXt[kTB * TW + c] = __ldg(a.X.b + i);
    }
  }
  for (int r = tid; r < TZ; r += blockDim.x) {
    const int k = z0 + r;
    const float ikh = __ldg(a.Z.ikh + k), adh = __ldg(a.Z.adh + k), ik = __ldg(a.Z.ik + k), ad = __ldg(a.Z.ad + k);
    sZt[kTKH * TZ + r] = ikh + adh;
    sZt[kTADH * TZ + r] = adh;
    sZt[kTBH * TZ + r] = __ldg(a.Z.bh + k);
    sZt[kTIKH * TZ + r] = ikh;
    sZt[kTK * TZ + r] = ik + ad;
    sZt[kTAD * TZ + r] = ad;
    sZt[kTB * TZ + r] = __ldg(a.Z.b + k);
  }

  // ---- load the cells
  float4 lx[RB], lz[RB], lh[RB];
  unsigned m[RB];
  unsigned zsb = 0;  // bit j: row j lies in the z-strip
  bool xs = false;
  int se = -1;       // 4 * row + element of the source cell
  unsigned mup = 0;  // bit e: cell e of the row above the thread's first row is in the H range
#pragma unroll
  for (int j = 0; j < RB; ++j) {
    lx[j] = lz[j] = lh[j] = zero4;
    m[j] = 0u;
  }
  bool fast = false;
  if (cell) {
    constexpr unsigned kPlain = (15u << kAEX) | (15u << kAEZ) | (15u << kAH) | (15u << kACELL);
    fast = true;
#pragma unroll
    for (int j = 0; j < RB; ++j) {
      if (j >= nrows) continue;
      const int row = rbase + j, k = z0 + row;
      const int gg = k * P + i0, so = 4 * (j * kResCellThreads + tid);
      lx[j] = ld4(a.Lx + gg);
      lz[j] = ld4(a.Lz + gg);
      lh[j] = ld4(a.Lh + gg);
      sts4(sCAx + so, ld4(a.CAx + gg));
      sts4(sCBx + so, ld4(a.CBx + gg));
      sts4(sCAz + so, ld4(a.CAz + gg));
      sts4(sCBz + so, ld4(a.CBz + gg));
      if (in_strip(k, NZ, W)) {
        zsb |= 1u << j;
        const int zrow = strip_idx(k, NZ, W) * P + i0;
        sts4(sLA + zoff(row), ld4(a.LA + zrow));
        sts4(sLC + zoff(row), ld4(a.LC + zrow));
      }
      unsigned mm = 0;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        if (i >= NX) continue;
        mm |= 1u << (kACELL + e);
        if (in_strip(i, NX, W)) {
          xs = true;
          mm |= 1u << (kAXS + e);
          const int q = k * (2 * W) + strip_idx(i, NX, W);
          sLB[xoff(row) + e] = a.LB[q];
          sLD[xoff(row) + e] = a.LD[q];
        }
        if (i <= NX - 2 && k >= 1 && k <= NZ - 2) mm |= 1u << (kAEX + e);
        if (k <= NZ - 2 && i >= 1 && i <= NX - 2) mm |= 1u << (kAEZ + e);
        if (i <= NX - 2 && k <= NZ - 2) mm |= 1u << (kAH + e);
        if (i == 0 || i == NX - 2 || k == 0 || k == NZ - 1) mm |= 1u << (kAXE + e);
        if (i == 0 || i == NX - 1 || k == 0 || k == NZ - 2) mm |= 1u << (kAZE + e);
        if (hy_plane(i, k, NX, NZ)) mm |= 1u << (kAHE + e);
        if (k == a.sk && i == a.si) se = 4 * j + e;
      }
      m[j] = mm;
      fast = fast && mm == kPlain;  // all four cells updated, none on a plane or a strip
    }
    fast = fast && zsb == 0 && se < 0 && i0 >= 4;
    const int ka = z0 + rbase - 1;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int i = i0 + e;
      if (ka >= 0 && i <= NX - 2 && ka <= NZ - 2) mup |= 1u << e;
    }
  }
  // receivers of this tile
  for (int q = tid; q < a.nrec; q += blockDim.x) {
    const int i = a.rec[3 * q], kk = a.rec[3 * q + 2];
    if (i >= x0 && i < x0 + nxt && kk >= z0 && kk < z0 + nzt) {
      const int pos = atomicAdd(&s_nrec, 1);
      if (pos < kResMaxLocalRec) {
        s_rec[2 * pos] = q;
        s_rec[2 * pos + 1] = (kk - z0) * TW + (i - x0);
      }
    }
  }
  __syncthreads();
  const int nloc = s_nrec;
  unsigned recm = 0;  // own cells that are receivers, bit 4 * row + element
  if (cell) {
    for (int q = 0; q < min(nloc, kResMaxLocalRec); ++q) {
      const int c = s_rec[2 * q + 1], row = c / TW, col = c - row * TW;
      if (row >= rbase && row < rbase + nrows && col >= 4 * tx && col < 4 * tx + 4)
        recm |= 1u << (4 * (row - rbase) + col - 4 * tx);
    }
    if (nloc > kResMaxLocalRec) {
      for (int q = 0; q < a.nrec; ++q) {
        const int i = a.rec[3 * q], kk = a.rec[3 * q + 2];
        if (i >= i0 && i < i0 + 4 && kk >= z0 + rbase && kk < z0 + rbase + nrows)
          recm |= 1u << (4 * (kk - z0 - rbase) + i - i0);
      }
    }
  }
  const float dbH = a.dbH;

  // dJ/d(trace) of step t into lam_Ex, lam_Ez of the receiver cells
  auto inject = [&](int t) {
    if (!recm) return;
    const float* rx = a.resid + (size_t)t * 2 * a.nrec;
#pragma unroll
    for (int j = 0; j < RB; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (!(recm & (1u << (4 * j + e)))) continue;
        const int c = (rbase + j) * TW + 4 * tx + e;
        float dx = 0.0f, dz = 0.0f;
        if (nloc <= kResMaxLocalRec) {
          for (int q = 0; q < nloc; ++q)
            if (s_rec[2 * q + 1] == c) {
              dx += rx[s_rec[2 * q]];
              dz += rx[a.nrec + s_rec[2 * q]];
            }
        } else {
          for (int q = 0; q < a.nrec; ++q)
            if (a.rec[3 * q] == i0 + e && a.rec[3 * q + 2] == z0 + rbase + j) {
              dx += rx[q];
              dz += rx[a.nrec + q];
            }
        }
        el(lx[j], e) += dx;
        el(lz[j], e) += dz;
      }
  };
  // gx of the thread's row j (zero outside the Ex range)
  auto gx_row = [&](int j) {
    float4 gx = zero4;
    const int row = rbase + j, so = 4 * (j * kResCellThreads + tid);
    const float4 cb = lds4(sCBx + so);
    const float kz = sZt[kTKH * TZ + row];
    const bool zs = (zsb >> j) & 1u;
    float4 lc = zero4;
    float adh = 0.0f;
    if (zs) {
      lc = lds4(sLC + zoff(row));
      adh = sZt[kTADH * TZ + row];
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      if (!mbit(m[j], kAEX, e)) continue;
      const float lex = mbit(m[j], kAXE, e) ? 0.0f : el(lx[j], e);
      float v = el(cb, e) * lex * kz;
      if (zs) v += el(lc, e) * adh;
      el(gx, e) = v;
    }
    return gx;
  };
  // gz of cell e of the thread's row j (zero outside the Ez range)
  auto gz_cell = [&](int j, int e) {
    if (!mbit(m[j], kAEZ, e)) return 0.0f;
    const int so = 4 * (j * kResCellThreads + tid);
    const float lez = mbit(m[j], kAZE, e) ? 0.0f : el(lz[j], e);
    float v = sCBz[so + e] * lez * sXt[kTKH * TW + 4 * tx + e];
    if (mbit(m[j], kAXS, e)) v += sLD[xoff(rbase + j) + e] * sXt[kTADH * TW + 4 * tx + e];
    return v;
  };
  // the first row's gx and every row's first gz, to the neighbours inside
  // the tile and, on the tile's edges, to the neighbouring tiles
  auto publish_g = [&](int par, unsigned tag) {
#pragma unroll
    for (int j = 0; j < RB; ++j) {
      if (j >= nrows) continue;
      const int row = rbase + j;
      const float v = gz_cell(j, 0);
      sGzCol[row * SX + tx] = v;
      if (left && tx == 0) ll_put1(ecol(par, 0, bx) + z0 + row, v, tag);
    }
    const float4 g0 = gx_row(0);
    sts4(sGxRow + ty * TW + 4 * tx, g0);
    if (up && rbase == 0) ll_put4(erow(par, 0, bz) + i0, g0, tag);
  };
  // Hy' of the row above the thread's first row (slot s + 1, step s0 + s)
  auto hy_above = [&](int s) {
    float4 h = zero4;
    if (mup) {
      const float4 hv = ld4(slot_f(a, s + 1, 2) + (size_t)(z0 + rbase - 1) * P + i0);
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if ((mup >> e) & 1u) el(h, e) = el(hv, e);
    }
    return h;
  };

  // the forward state phase A of slot s reads, into this thread's staging slots
  auto stage = [&](int s) {
    const float *SEx = slot_f(a, s, 0), *SEz = slot_f(a, s, 1), *S1Hy = slot_f(a, s + 1, 2);
#pragma unroll
    for (int j = 0; j < RB; ++j) {
      if (j >= nrows) continue;
      const size_t gg = (size_t)(z0 + rbase + j) * P + i0;
      const int so = 4 * (j * kResCellThreads + tid);
      cp_async16(sSEx + so, SEx + gg);
      cp_async16(sSEz + so, SEz + gg);
      cp_async16(sSHy + so, S1Hy + gg);
    }
  };

  if (cell) {
    stage(a.nsteps - 1);
    inject(a.s0 + a.nsteps - 1);
    publish_g(0, 1u);
  } else if (xwarp) {  // gx row below and gz column to the right for the first transposed step
    if (!fetch_edges(down ? erow(0, 0, bz + 1) + x0 : nullptr, sGxRow + TYT * TW, down ? TW : 0,
                     right ? ecol(0, 0, bx + 1) + z0 : nullptr, sGzCol + TXT, SX, right ? nzt : 0, 1u, ctl,
                     a.limit_ns) &&
        (tid & 31) == 0)
      s_abort = 1;
  }
  __syncthreads();

  float acc0 = 0.0f, acc1 = 0.0f;  // source terms of this sweep
  bool ok = s_abort == 0;
  for (int it = 0; it < a.nsteps && ok; ++it) {
    const int s = a.nsteps - 1 - it;  // slot of the state before step t
    const int t = a.s0 + s;
    const int par = it & 1;
    const unsigned tag = (unsigned)it + 1u;

    // ================= phase A: E half transposed, gradients, source
    if (cell) cp_async_wait_all();  // this step's staged forward state
    if (cell && fast) {  // interior cells: no masks, no strips
      const float* S1Hy = slot_f(a, s + 1, 2);
      float4 sx[RB], sz[RB], h1[RB];
      float hl[RB];
#pragma unroll
      for (int j = 0; j < RB; ++j) {
        sx[j] = sz[j] = h1[j] = zero4;
        hl[j] = 0.0f;
        if (j >= nrows) continue;
        const int gg = (z0 + rbase + j) * P + i0;
        const int so = 4 * (j * kResCellThreads + tid);
        sx[j] = lds4(sSEx + so);
        sz[j] = lds4(sSEz + so);
        h1[j] = lds4(sSHy + so);
        hl[j] = __ldg(S1Hy + gg - 1);
      }
      float4 hpm = hy_above(s);
      const float4 khx = lds4(sXt + kTKH * TW + 4 * tx), ikhx = lds4(sXt + kTIKH * TW + 4 * tx);
      const float kx3 = sXt[kTK * TW + 4 * tx + 3];
      float4 gcur = lds4(sGxRow + ty * TW + 4 * tx);
#pragma unroll
      for (int j = 0; j < RB; ++j) {
        if (j >= nrows) continue;
        const int row = rbase + j, k = z0 + row, so = 4 * (j * kResCellThreads + tid);
        float4 gnext;
        if (j + 1 < RB && j + 1 < nrows) {
          const int jn = j + 1 < RB ? j + 1 : j;
          const float4 cb = lds4(sCBx + so + 4 * kResCellThreads);
          const float kz = sZt[kTKH * TZ + row + 1];
#pragma unroll
          for (int e = 0; e < 4; ++e) el(gnext, e) = el(cb, e) * el(lx[jn], e) * kz;
        } else {
          gnext = lds4(sGxRow + (ty + 1) * TW + 4 * tx);
        }
        const float4 cbz = lds4(sCBz + so);
        float gz[5];
        gz[0] = sGzCol[row * SX + tx];
#pragma unroll
        for (int e = 1; e < 4; ++e) gz[e] = el(cbz, e) * el(lz[j], e) * el(khx, e);
        gz[4] = sGzCol[row * SX + tx + 1];
        const float4 cax = lds4(sCAx + so), caz = lds4(sCAz + so);
        float4 gax = lds4(sGAx + so), gbx = lds4(sGBx + so), gaz = lds4(sGAz + so), gbz = lds4(sGBz + so);
        const float ikhz = sZt[kTIKH * TZ + row];
        const float4 hp = h1[j];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const float lex = el(lx[j], e), lez = el(lz[j], e);
          el(gax, e) += lex * el(sx[j], e);
          el(gbx, e) += lex * ((el(hp, e) - el(hpm, e)) * ikhz);
          el(gaz, e) += lez * el(sz[j], e);
          el(gbz, e) += lez * ((el(hp, e) - (e == 0 ? hl[j] : el(hp, e > 0 ? e - 1 : 0))) * el(ikhx, e));
          el(lh[j], e) = el(lh[j], e) + el(gcur, e) - el(gnext, e) + gz[e] - gz[e + 1];
          el(lx[j], e) = el(cax, e) * lex;
          el(lz[j], e) = el(caz, e) * lez;
        }
        sts4(sGAx + so, gax);
        sts4(sGBx + so, gbx);
        sts4(sGAz + so, gaz);
        sts4(sGBz + so, gbz);
        const float4 th = lh[j];
        if (j == RB - 1 || (down && row == nzt - 1)) {
          const float kz = sZt[kTK * TZ + row];
          float4 ha;
#pragma unroll
          for (int e = 0; e < 4; ++e) el(ha, e) = dbH * el(th, e) * kz;
          if (j == RB - 1) sts4(sHaRow + (ty + 1) * TW + 4 * tx, ha);
          if (down && row == nzt - 1) ll_put4(erow(par, 1, bz) + i0, ha, tag);
        }
        const float hb3 = dbH * th.w * kx3;
        sHbCol[row * SX + tx + 1] = hb3;
        if (right && tx == TXT - 1) ll_put1(ecol(par, 1, bx) + k, hb3, tag);
        gcur = gnext;
        hpm = hp;
      }
    } else if (cell) {  // strip, plane, source or partial groups: per-cell masks
      const float* S1Hy = slot_f(a, s + 1, 2);
      float4 gcur = lds4(sGxRow + ty * TW + 4 * tx);
      float4 hpm = hy_above(s);
#pragma unroll
      for (int j = 0; j < RB; ++j) {
        if (j >= nrows) continue;
        const int row = rbase + j, k = z0 + row;
        const int gg = k * P + i0, so = 4 * (j * kResCellThreads + tid);
        const unsigned mj = m[j];
        const bool zs = (zsb >> j) & 1u;
        float4 gnext;
        if (j + 1 < RB && j + 1 < nrows) gnext = gx_row(j + 1 < RB ? j + 1 : j);
        else gnext = lds4(sGxRow + (ty + 1) * TW + 4 * tx);
        float gz[5];
        gz[0] = sGzCol[row * SX + tx];
        {
          const float4 cbz = lds4(sCBz + so), khx = lds4(sXt + kTKH * TW + 4 * tx);
          float4 ld = zero4, adhx = zero4;
          if (xs) {
            ld = lds4(sLD + xoff(row));
            adhx = lds4(sXt + kTADH * TW + 4 * tx);
          }
#pragma unroll
          for (int e = 1; e < 4; ++e) {
            float v = 0.0f;
            if (mbit(mj, kAEZ, e)) {
              const float lez = mbit(mj, kAZE, e) ? 0.0f : el(lz[j], e);
              v = el(cbz, e) * lez * el(khx, e);
              if (mbit(mj, kAXS, e)) v += el(ld, e) * el(adhx, e);
            }
            gz[e] = v;
          }
        }
        gz[4] = sGzCol[row * SX + tx + 1];
        // Hy' of the row and of the cell on the left
        const float4 h1 = lds4(sSHy + so);
        float4 hp;
#pragma unroll
        for (int e = 0; e < 4; ++e)
          el(hp, e) = mbit(mj, kAH, e) ? el(h1, e) : 0.0f;
        const float hpl = (i0 >= 1 && k <= NZ - 2) ? __ldg(S1Hy + gg - 1) : 0.0f;
        // Ex: gradients and lam_C
        {
          const float4 sx = lds4(sSEx + so), cax = lds4(sCAx + so), cbx = lds4(sCBx + so);
          float4 gax = lds4(sGAx + so), gbx = lds4(sGBx + so);
          const float ikhz = sZt[kTIKH * TZ + row];
          float4 lc = zero4, s1c = zero4;
          float bhz = 0.0f;
          if (zs) {
            lc = lds4(sLC + zoff(row));
            s1c = ld4(slot_f(a, s + 1, 5) + (size_t)strip_idx(k, NZ, W) * P + i0);
            bhz = sZt[kTBH * TZ + row];
          }
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const float lex = mbit(mj, kAXE, e) ? 0.0f : el(lx[j], e);
            float mx = lex;
            if (mbit(mj, kAEX, e)) {
              mx = el(cax, e) * lex;
              float d = (el(hp, e) - el(hpm, e)) * ikhz;
              if (zs) {
                d += el(s1c, e);
                el(lc, e) = bhz * (el(cbx, e) * lex + el(lc, e));
              }
              el(gax, e) += lex * el(sx, e);
              el(gbx, e) += lex * d;
            }
            if (4 * j + e == se) acc0 += lex * __ldg(a.srcfn + t);
            // TH, with the gx of this row and of the row below
            const float lhy = mbit(mj, kAHE, e) ? 0.0f : el(lh[j], e);
            el(lh[j], e) = lhy + el(gcur, e) - el(gnext, e) + gz[e] - gz[e + 1];
            el(lx[j], e) = mx;
          }
          sts4(sGAx + so, gax);
          sts4(sGBx + so, gbx);
          if (zs) sts4(sLC + zoff(row), lc);
        }
        // Ez: gradients and lam_D
        {
          const float4 sz = lds4(sSEz + so), caz = lds4(sCAz + so), cbz = lds4(sCBz + so);
          float4 gaz = lds4(sGAz + so), gbz = lds4(sGBz + so);
          const float4 ikhx = lds4(sXt + kTIKH * TW + 4 * tx);
          float4 ld = zero4, s1d = zero4, bhx = zero4;
          if (xs) {
            ld = lds4(sLD + xoff(row));
            bhx = lds4(sXt + kTBH * TW + 4 * tx);
            const float* S1D = slot_f(a, s + 1, 6) + (size_t)k * (2 * W);
#pragma unroll
            for (int e = 0; e < 4; ++e)
              if (mbit(mj, kAXS, e)) el(s1d, e) = __ldg(S1D + strip_idx(i0 + e, NX, W));
          }
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const float lez = mbit(mj, kAZE, e) ? 0.0f : el(lz[j], e);
            float mz = lez;
            if (mbit(mj, kAEZ, e)) {
              mz = el(caz, e) * lez;
              float d = (el(hp, e) - (e == 0 ? hpl : el(hp, e > 0 ? e - 1 : 0))) * el(ikhx, e);
              if (mbit(mj, kAXS, e)) {
                d += el(s1d, e);
                el(ld, e) = el(bhx, e) * (el(cbz, e) * lez + el(ld, e));
              }
              el(gaz, e) += lez * el(sz, e);
              el(gbz, e) += lez * d;
            }
            if (4 * j + e == se) acc1 += lez * __ldg(a.srcfn + a.nstep + t);
            el(lz[j], e) = mz;
          }
          sts4(sGAz + so, gaz);
          sts4(sGBz + so, gbz);
          if (xs) sts4(sLD + xoff(row), ld);
        }
        // hA of the last row and hB of the last column, for phase B of the neighbours
        {
          const float4 th = lh[j];
          float4 la = zero4;
          float adz = 0.0f;
          if (zs) {
            la = lds4(sLA + zoff(row));
            adz = sZt[kTAD * TZ + row];
          }
          if (j == RB - 1 || (down && row == nzt - 1)) {
            const float kz = sZt[kTK * TZ + row];
            float4 ha = zero4;
#pragma unroll
            for (int e = 0; e < 4; ++e)
              if (mbit(mj, kAH, e)) el(ha, e) = dbH * el(th, e) * kz + (zs ? el(la, e) * adz : 0.0f);
            if (j == RB - 1) sts4(sHaRow + (ty + 1) * TW + 4 * tx, ha);
            if (down && row == nzt - 1) ll_put4(erow(par, 1, bz) + i0, ha, tag);
          }
          float hb3 = 0.0f;
          if (mbit(mj, kAH, 3)) {
            hb3 = dbH * th.w * sXt[kTK * TW + 4 * tx + 3];
            if (mbit(mj, kAXS, 3)) hb3 += sLB[xoff(row) + 3] * sXt[kTAD * TW + 4 * tx + 3];
          }
          sHbCol[row * SX + tx + 1] = hb3;
          if (right && tx == TXT - 1) ll_put1(ecol(par, 1, bx) + k, hb3, tag);
        }
        gcur = gnext;
        hpm = hp;
      }
    } else if (xwarp) {  // hA row above and hB column on the left for phase B
      if (!fetch_edges(up ? erow(par, 1, bz - 1) + x0 : nullptr, sHaRow, up ? TW : 0,
                       left ? ecol(par, 1, bx - 1) + z0 : nullptr, sHbCol, SX, left ? nzt : 0, tag, ctl,
                       a.limit_ns) &&
          (tid & 31) == 0)
        s_abort = 1;
    }
    __syncthreads();
    if (s_abort) {
      ok = false;
      break;
    }

    // ================= phase B: H half transposed
    if (cell) {
      if (it + 1 < a.nsteps) {  // the forward state of the next transposed step: staged, strips into L2
        stage(s - 1);
#pragma unroll
        for (int j = 0; j < RB; ++j) {
          if (j >= nrows) continue;
          const int k = z0 + rbase + j;
          if ((zsb >> j) & 1u) prefetch_l2(slot_f(a, s, 5) + strip_idx(k, NZ, W) * P + i0);
          if (xs) {
#pragma unroll
            for (int e = 0; e < 4; ++e)
              if (mbit(m[j], kAXS, e)) prefetch_l2(slot_f(a, s, 6) + k * (2 * W) + strip_idx(i0 + e, NX, W));
          }
        }
      }
      float4 hAm = lds4(sHaRow + ty * TW + 4 * tx);
      const float4 kx = lds4(sXt + kTK * TW + 4 * tx);
      if (fast) {
#pragma unroll
        for (int j = 0; j < RB; ++j) {
          if (j >= nrows) continue;
          const int row = rbase + j;
          const float4 th = lh[j];
          const float kz = sZt[kTK * TZ + row];
          float4 ha;
          float hb[5];
          hb[0] = sHbCol[row * SX + tx];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            el(ha, e) = dbH * el(th, e) * kz;
            hb[e + 1] = dbH * el(th, e) * el(kx, e);
          }
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            el(lx[j], e) = el(lx[j], e) + el(hAm, e) - el(ha, e);
            el(lz[j], e) = el(lz[j], e) + hb[e] - hb[e + 1];
          }
          hAm = ha;
        }
      } else {
#pragma unroll
        for (int j = 0; j < RB; ++j) {
          if (j >= nrows) continue;
          const int row = rbase + j;
          const unsigned mj = m[j];
          const bool zs = (zsb >> j) & 1u;
          const float4 th = lh[j];
          const float kz = sZt[kTK * TZ + row];
          float4 la = zero4;
          float adz = 0.0f, bzz = 0.0f;
          if (zs) {
            la = lds4(sLA + zoff(row));
            adz = sZt[kTAD * TZ + row];
            bzz = sZt[kTB * TZ + row];
          }
          float4 ha = zero4;
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (mbit(mj, kAH, e)) el(ha, e) = dbH * el(th, e) * kz + (zs ? el(la, e) * adz : 0.0f);
          float4 lb = zero4, adx = zero4, bxx = zero4;
          if (xs) {
            lb = lds4(sLB + xoff(row));
            adx = lds4(sXt + kTAD * TW + 4 * tx);
            bxx = lds4(sXt + kTB * TW + 4 * tx);
          }
          float hb[5];
          hb[0] = sHbCol[row * SX + tx];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            float v = 0.0f;
            if (mbit(mj, kAH, e)) {
              v = dbH * el(th, e) * el(kx, e);
              if (mbit(mj, kAXS, e)) v += el(lb, e) * el(adx, e);
            }
            hb[e + 1] = v;
          }
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const bool on = mbit(mj, kACELL, e), hr = mbit(mj, kAH, e);
            el(lx[j], e) = on ? el(lx[j], e) + el(hAm, e) - el(ha, e) : 0.0f;
            el(lz[j], e) = on ? el(lz[j], e) + hb[e] - hb[e + 1] : 0.0f;
            el(lh[j], e) = (!on || (hr && mbit(mj, kAHE, e))) ? 0.0f : el(th, e);
            if (hr && mbit(mj, kAXS, e)) el(lb, e) = el(bxx, e) * (dbH * el(th, e) + el(lb, e));
            if (hr && zs) el(la, e) = bzz * (dbH * el(th, e) + el(la, e));
          }
          if (zs) sts4(sLA + zoff(row), la);
          if (xs) sts4(sLB + xoff(row), lb);
          hAm = ha;
        }
      }
      if (it + 1 < a.nsteps) {
        inject(t - 1);
        publish_g(par ^ 1, tag + 1u);
      }
    } else if (xwarp && it + 1 < a.nsteps) {  // gx row below and gz column to the right for the next step
      if (!fetch_edges(down ? erow(par ^ 1, 0, bz + 1) + x0 : nullptr, sGxRow + TYT * TW, down ? TW : 0,
                       right ? ecol(par ^ 1, 0, bx + 1) + z0 : nullptr, sGzCol + TXT, SX, right ? nzt : 0,
                       tag + 1u, ctl, a.limit_ns) &&
          (tid & 31) == 0)
        s_abort = 1;
    }
    __syncthreads();
    if (s_abort) ok = false;
  }
  cp_async_wait_all();  // no copy left in flight
  if (!ok) return;  // the adjoint state is left as it was loaded; the host reports the timeout

  // ---- write the adjoint state back, add the gradient sums
  if (cell) {
#pragma unroll
    for (int j = 0; j < RB; ++j) {
      if (j >= nrows) continue;
      const int row = rbase + j, k = z0 + row;
      const int gg = k * P + i0, so = 4 * (j * kResCellThreads + tid);
      st4(a.Lx + gg, lx[j]);
      st4(a.Lz + gg, lz[j]);
      st4(a.Lh + gg, lh[j]);
      if ((zsb >> j) & 1u) {
        const int zrow = strip_idx(k, NZ, W) * P + i0;
        st4(a.LA + zrow, lds4(sLA + zoff(row)));
        st4(a.LC + zrow, lds4(sLC + zoff(row)));
      }
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (mbit(m[j], kAXS, e)) {
          const int q = k * (2 * W) + strip_idx(i0 + e, NX, W);
          a.LB[q] = sLB[xoff(row) + e];
          a.LD[q] = sLD[xoff(row) + e];
        }
      float* gp[4] = {a.gCAx, a.gCBx, a.gCAz, a.gCBz};
      const float* gs[4] = {sGAx, sGBx, sGAz, sGBz};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        float4 v = *reinterpret_cast<const float4*>(gp[q] + gg);
        const float4 d = lds4(gs[q] + so);
        v.x += d.x;
        v.y += d.y;
        v.z += d.z;
        v.w += d.w;
        st4(gp[q] + gg, v);
      }
    }
    if (se >= 0) {
      atomicAdd(a.srcacc, acc0);
      atomicAdd(a.srcacc + 1, acc1);
    }
  }
}

}  // namespace

size_t em2_adj_resident_smem(const ResPlan& plan, int NX, int NZ, int W) {
  size_t m = 0;
  for (int b = 0; b < plan.ntiles; ++b) {
    const int4 t = plan.tile[b];
    const int x0 = t.x & 0xffff, z0 = t.y & 0xffff;
    const int TW = (((t.x >> 16) - x0) + 3) & ~3, TZ = (t.y >> 16) - z0;
    int nzr, nxg;
    adj_tile_strips(x0, TW, z0, TZ, NX, NZ, W, &nzr, &nxg);
    const size_t SX = (size_t)TW / 4 + 1, TYT = ((size_t)TZ + kResRows - 1) / kResRows, CS = 4 * (size_t)kResRows * kResCellThreads;
    m = std::max(m, sizeof(float) * (11 * CS + 2 * (size_t)nzr * TW + 8 * (size_t)TZ * nxg + 2 * (TYT + 1) * TW +
                                     kNT * (size_t)TW + kNT * (size_t)TZ + 2 * (size_t)TZ * SX));
  }
  return m;
}

cudaError_t em2_adj_resident_prepare(const ResPlan& plan, int NX, int NZ, int W, int* ctas_per_sm) {
  *ctas_per_sm = 0;
  const size_t smem = em2_adj_resident_smem(plan, NX, NZ, W);
  cudaError_t e = res_allow_max_smem((const void*)em2_adj_resident_kernel);
  if (e != cudaSuccess) return e;
  // ask for no more shared memory than the largest tile needs, so the rest of
  // the SM's on-chip memory serves as L1 (it holds the kernel's register spills)
  int dev = 0, per_sm = 0;
  cudaFuncAttributes fa;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, em2_adj_resident_kernel);
  if (e != cudaSuccess) return e;
  const size_t need = smem + fa.sharedSizeBytes + 1024;  // the runtime reserves 1 KB per CTA
  const int pct = (int)std::min<size_t>(100, (100 * need + per_sm - 1) / per_sm);
  e = cudaFuncSetAttribute(em2_adj_resident_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, em2_adj_resident_kernel, kResThreads, smem);
}

cudaError_t em2_adj_resident_launch(const Em2AdjResident& a, cudaStream_t s) {
  void* args[] = {(void*)&a};
  return cudaLaunchCooperativeKernel((const void*)em2_adj_resident_kernel, dim3(a.plan.ntiles), dim3(kResThreads), args,
                                     em2_adj_resident_smem(a.plan, a.NX, a.NZ, a.W), s);
}

}  // namespace sfd
