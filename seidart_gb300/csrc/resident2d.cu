// SM-resident electromag2 run: every time step of an sfd_run in one
// cooperative launch, with the whole state on chip.
//
// Tile (bx, bz) of TW x TZ cells (ResPlan) belongs to one CTA for the whole run.  Cell
// thread (tx, ty) owns the cells 4tx..4tx+3 of tile row ty and keeps their
// Ex, Ez and Hy in registers from the first step to the last; the update
// coefficients and the CPML memory variables stay in shared memory.  The per-cell arithmetic is that of the single-pass tile
// (fused2d.cuh), i.e. the loops of legacy/fortran/electromagfdtd.f95:249-321,
// so the streaming and on-chip forms give the same fields.
//
// Inside a tile, the values a thread needs from its neighbours pass through
// four shared-memory arrays:
//   H half-step: Hy(i,k) needs Ex(i,k+1) -- the row of the thread below
//     (sExRow) -- and Ez(i+4,k) -- the first column of the thread to the right
//     (sEzCol);
//   E half-step: Ex(i,k) needs Hy(i,k-1) -- the row of the thread above
//     (sHyRow) -- and Ez(i,k) needs Hy(i-1,k) -- the last column of the thread
//     to the left (sHyCol).
// Between tiles the same edges travel through global memory (L2) as 8-byte
// words {value, tag} (resident.h), tag = s + 1 for the step s that reads
// them, in the copy of parity s & 1.  Cell threads on a tile edge write their
// words as soon as they are computed; the last warp of the CTA polls the
// neighbours' words during each half-step and copies them into the halo
// entries of those arrays (row TZ, column TXT, row 0, column 0) before the
// barrier that ends the half-step.  A tile can be at most one step ahead of a neighbour
// that reads its edges, so two copies keep a word from being overwritten
// before it is read.  The polling warp gives up after limit_ns (%globaltimer)
// or when another tile has given up, records the failure in the control block,
// and the CTA leaves the run at the next barrier; the host reports
// SFD_ERR_TIMEOUT.  The launch is cooperative, so all tiles are co-resident
// and a correct run never reaches the limit.
//
// Threads whose four cells are away from the CPML strips, the Dirichlet
// planes and the source take a short path; the others apply the strip
// recursions and, through per-cell masks fixed at the start, the loop bounds,
// Dirichlet planes and source of the Fortran -- the same operations in the
// same order.
#include <algorithm>
#include <vector>

#include "resident_common.cuh"

namespace sfd {

using namespace res;

namespace {

// One CTA's tile for the whole run.  MODE 0: a run; 1: a recompute for the
// adjoint (every step's state dumped, the handle's state kept); 2: a run that
// also saves checkpoints.  RB rows per thread: kResRows in general, kResRows3
// in the tiles the planner marks as interior (no CPML strip cell, no
// Dirichlet plane; the source may lie inside), which take the short update
// path only and so hold half as many cells again per thread.
template <int MODE, int RB>
__device__ __forceinline__ void em2_resident_tile(const Em2Resident& a, float* smem, int& s_abort, int& s_nrec,
                                                  int* s_rec) {
  constexpr bool DUMP = MODE == 1, CKPT = MODE == 2;
  constexpr bool INTERIOR = RB == kResRows3;
  const int NX = a.NX, NZ = a.NZ, P = a.P, W = a.W;
  const int tile = blockIdx.x;
  const int4 te = a.plan.tile[tile];
  const int x0 = te.x & 0xffff, z0 = te.y & 0xffff, bz = te.z & 0xffff, bx = te.z >> 16;
  const int nxt = (te.x >> 16) - x0, nzt = (te.y >> 16) - z0;
  const int TW = (nxt + 3) & ~3, TZ = nzt;  // this tile's shared-memory layout
  const int TXT = TW >> 2, TYT = (TZ + RB - 1) / RB, SX = TXT + 1;
  const int nc4 = TXT;
  // row edges are indexed by tile row and global x, column edges by the index
  // in the tile row and global z, so a tile row may be cut unlike its neighbours
  const bool up = bz > 0, down = bz < a.plan.ntz - 1, left = bx > 0, right = bx < (te.w & 0xffff) - 1;
  const int tid = threadIdx.x;
  const bool xwarp = tid >= kResCellThreads;
  // Threads take the tile's groups (four columns x RB rows) in class order --
  // interior groups on a side that has a neighbour tile, the other interior
  // groups, CPML strip groups, then groups with a boundary plane or the
  // source -- so each warp runs one update path instead of several in turn,
  // and the edge words the neighbours wait for come from the first warps
  // (4 % fewer us per step on the 1040 x 540 grid than interior groups in
  // row order).
  const int ngroups = TXT * TYT;
  int cls = 4;
  if (!xwarp && tid < ngroups) {
    const int gi = x0 + 4 * (tid % TXT), gk0 = z0 + RB * (tid / TXT);
    const int gk1 = min(gk0 + RB, z0 + nzt) - 1;
    const bool edge = gi < 1 || gi + 3 > NX - 3 || gk0 < 1 || gk1 > NZ - 3 ||
                      (a.io.sk >= gk0 && a.io.sk <= gk1 && a.io.si >= gi && a.io.si < gi + 4);
    const bool strp = in_strip(gk0, NZ, W) || in_strip(gk1, NZ, W) || in_strip(gi, NX, W) || in_strip(gi + 3, NX, W);
    const int tx0 = tid % TXT, ty0 = tid / TXT;
    const bool perim = (up && ty0 == 0) || (down && ty0 == TYT - 1) || (left && tx0 == 0) || (right && tx0 == TXT - 1);
    cls = edge ? 3 : (strp ? 2 : (perim ? 0 : 1));
  }
  const int g = class_ordered_group<4>(cls);
  const int tx = g >= 0 ? g % TXT : 0, ty = g >= 0 ? g / TXT : 0;
  const int rbase = RB * ty;
  const int nrows = g >= 0 ? min(RB, nzt - rbase) : 0;
  const bool cell = nrows > 0;
  const int i0 = x0 + 4 * tx;
  // Arrays only the owning thread reads are indexed by thread: row j of
  // thread tid is the float4 at so = 4 (j * kResCellThreads + tid), so a warp's
  // accesses are conflict-free whichever groups its threads own.
  const int CS = 4 * RB * kResCellThreads;
  constexpr int NPSI = INTERIOR ? 0 : 4;  // an interior tile has no memory variables
  float* sMExz = smem;  // CPML memory variables of strip cells
  float* sMEzx = sMExz + CS;
  float* sMHyz = sMEzx + CS;
  float* sMHyx = sMHyz + CS;
  float* sCAx = smem + NPSI * CS;  // update coefficients
  float* sCBx = sCAx + CS;
  float* sCAz = sCBx + CS;
  float* sCBz = sCAz + CS;
  float* sExRow = sCBz + CS;                // [TYT+1][TW]: first Ex row of thread row ty; row TYT = tile below
  float* sHyRow = sExRow + (TYT + 1) * TW;  // [TYT+1][TW]: row ty+1 = last Hy row of thread row ty; row 0 = tile above
  // scalar arrays last: every array above starts on a 16-byte boundary (TW is a multiple of 4)
  float* sEzCol = sHyRow + (TYT + 1) * TW;  // [TZ][SX]: first Ez column of thread column tx; column TXT = tile right
  float* sHyCol = sEzCol + TZ * SX;         // [TZ][SX]: column tx+1 = last Hy column of tx; column 0 = tile left
  const int nsm = (NPSI + 4) * CS + 2 * (TYT + 1) * TW + 2 * TZ * SX;
  const int NZp = a.r.NZp;
  // edge words: field 0 = first Ex row / first Ez column, 1 = last Hy row / column
  auto erow = [&](int par, int f, int b) { return a.r.erow + (size_t)((par * 2 + f) * kResMaxTiles1D + b) * P; };
  auto ecol = [&](int par, int f, int b) { return a.r.ecol + (size_t)((par * 2 + f) * kResMaxTiles1D + b) * NZp; };
  Ctl* ctl = a.io.ctl;
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);

  for (int q = tid; q < nsm; q += blockDim.x) smem[q] = 0.0f;
  if (tid == 0) {
    s_nrec = 0;
    s_abort = 0;
  }
  __syncthreads();

  // ---- load the cells into registers
  float4 ex[RB], ez[RB], hy[RB];
  float ikz[RB], ikzh[RB];
  unsigned m[RB];  // per-row cell masks
  bool zs[RB];
  float4 ikx4 = zero4, ikxh4 = zero4;
  bool fast = false, plain = false, xs = false;
  int se = -1;  // 4 * row + element of the source cell
#pragma unroll
  for (int j = 0; j < RB; ++j) {
    ex[j] = ez[j] = hy[j] = zero4;
    ikz[j] = ikzh[j] = 0.0f;
    m[j] = 0u;
    zs[j] = false;
  }
  if (cell) {
    ikx4 = ld4(a.X.ik + i0);
    ikxh4 = ld4(a.X.ikh + i0);
    plain = true;
#pragma unroll
    for (int j = 0; j < RB; ++j) {
      if (j >= nrows) continue;
      const int row = rbase + j, k = z0 + row;
      const int gg = k * P + i0, so = 4 * (j * kResCellThreads + tid);
      ex[j] = ld4(a.Ex + gg);
      ez[j] = ld4(a.Ez + gg);
      hy[j] = ld4(a.Hy + gg);
      sts4(sCAx + so, ld4(a.CAx + gg));
      sts4(sCBx + so, ld4(a.CBx + gg));
      sts4(sCAz + so, ld4(a.CAz + gg));
      sts4(sCBz + so, ld4(a.CBz + gg));
      ikz[j] = __ldg(a.Z.ik + k);
      ikzh[j] = __ldg(a.Z.ikh + k);
      zs[j] = !INTERIOR && in_strip(k, NZ, W);
      if (zs[j]) {
        const int zrow = strip_idx(k, NZ, W) * P + i0;
        sts4(sMExz + so, ld4(a.mExz + zrow));
        sts4(sMHyz + so, ld4(a.mHyz + zrow));
      }
      unsigned mm = 0;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        if (i >= NX) continue;
        mm |= 1u << (kMCELL + e);
        if (!INTERIOR && in_strip(i, NX, W)) {
          xs = true;
          const int q = k * (2 * W) + strip_idx(i, NX, W);
          sMEzx[so + e] = a.mEzx[q];
          sMHyx[so + e] = a.mHyx[q];
        }
        if (i <= NX - 2 && k <= NZ - 2) mm |= 1u << (kMH + e);
        if (i <= NX - 2 && k >= 1 && k <= NZ - 2) mm |= 1u << (kMEX + e);
        if (k <= NZ - 2 && i >= 1 && i <= NX - 2) mm |= 1u << (kMEZ + e);
        if (i == 0 || i == NX - 2 || k == 0 || k == NZ - 1) mm |= 1u << (kMEXZ + e);
        if (i == 0 || i == NX - 1 || k == 0 || k == NZ - 2) mm |= 1u << (kMEZZ + e);
        if (i <= NX - 2 && k <= NZ - 2 && (i == 0 || i == NX - 2 || k == 0 || k == NZ - 2)) mm |= 1u << (kMHYZ + e);
        if (k == a.io.sk && i == a.io.si) se = 4 * j + e;
      }
      m[j] = mm;
      // all four cells updated, none on a Dirichlet plane
      plain = plain && (mm & 0xffffffu) == 0x000fffu;
      sEzCol[row * SX + tx] = ez[j].x;
      if (left && tx == 0) ll_put1(ecol(0, 0, bx) + k, ez[j].x, 1u);
    }
    plain = plain && se < 0;  // ... nor the source
    bool anyzs = false;
#pragma unroll
    for (int j = 0; j < RB; ++j) anyzs |= zs[j];
    fast = plain && !xs && !anyzs;  // and none in a strip
    sts4(sExRow + ty * TW + 4 * tx, ex[0]);
    if (up && rbase == 0) ll_put4(erow(0, 0, bz) + i0, ex[0], 1u);
  }
  // receivers of this tile
  for (int q = tid; q < a.io.nrec; q += blockDim.x) {
    const int i = a.io.rec[3 * q], kk = a.io.rec[3 * q + 2];
    if (i >= x0 && i < x0 + nxt && kk >= z0 && kk < z0 + nzt) {
      const int pos = atomicAdd(&s_nrec, 1);
      if (pos < kResMaxLocalRec) {
        s_rec[2 * pos] = q;
        s_rec[2 * pos + 1] = (kk - z0) * TW + (i - x0);
      }
    }
  }
  if (xwarp) {  // edges of the tiles below and to the right for step 0
    if (!fetch_edges(down ? erow(0, 0, bz + 1) + x0 : nullptr, sExRow + TYT * TW, down ? 4 * nc4 : 0,
                     right ? ecol(0, 0, bx + 1) + z0 : nullptr, sEzCol + TXT, SX, right ? nzt : 0, 1u + a.tag_bias, ctl,
                     a.limit_ns) &&
        (tid & 31) == 0)
      s_abort = 1;
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
      for (int q = 0; q < a.io.nrec; ++q) {
        const int i = a.io.rec[3 * q], kk = a.io.rec[3 * q + 2];
        if (i >= i0 && i < i0 + 4 && kk >= z0 + rbase && kk < z0 + rbase + nrows)
          recm |= 1u << (4 * (kk - z0 - rbase) + i - i0);
      }
    }
  }
  const float dbH = a.dbH;
  const bool hsrc = se >= 0;

  float nrm = 0.0f;
  bool ok = s_abort == 0;
  for (int s = 0; s < a.nsteps && ok; ++s) {
    const int t = a.t0 + s;
    const int par = s & 1;
    const unsigned tag = (unsigned)s + 1u;

    // ================= H half-step (electromagfdtd.f95:249-262)
    if (cell) {
      const float4 exb = lds4(sExRow + (ty + 1) * TW + 4 * tx);
#pragma unroll
      for (int j = 0; j < RB; ++j) {
        if (j >= nrows) continue;
        const int row = rbase + j, k = z0 + row, so = 4 * (j * kResCellThreads + tid);
        float4 exn = exb;
        if (j + 1 < RB && j + 1 < nrows) exn = ex[j + 1 < RB ? j + 1 : j];
        const float ezn = sEzCol[row * SX + tx + 1];
        float4 hv;
        if (INTERIOR || fast) {
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const float dEx = el(exn, e) - el(ex[j], e);
            const float dEz = (e < 3 ? el(ez[j], e + 1) : ezn) - el(ez[j], e);
            el(hv, e) = el(hy[j], e) + dbH * (dEz * el(ikx4, e) + dEx * ikz[j]);
          }
        } else if constexpr (!INTERIOR) {  // strip, bound or plane cells: two cells at a time, masks applied as selects
          const unsigned mj = m[j];
          const bool hall = ((mj >> kMH) & 15u) == 15u;
          float adz = 0.0f, bzc = 0.0f;
          if (zs[j]) {
            adz = __ldg(a.Z.ad + k);
            bzc = __ldg(a.Z.b + k);
          }
#pragma unroll
          for (int hh = 0; hh < 2; ++hh) {
            float2 pz = make_float2(0.f, 0.f), px = pz, adx = pz, bxx = pz;
            if (zs[j]) pz = lds2(sMExz + so + 2 * hh);
            if (xs) {
              px = lds2(sMEzx + so + 2 * hh);
              adx = ld2(a.X.ad + i0 + 2 * hh);
              bxx = ld2(a.X.b + i0 + 2 * hh);
            }
#pragma unroll
            for (int q = 0; q < 2; ++q) {
              const int e = 2 * hh + q;
              const bool on = hall || mbit(mj, kMH, e);
              const float dEx = el(exn, e) - el(ex[j], e);
              float vz = dEx * ikz[j];
              if (zs[j]) {
                const float p = bzc * el2(pz, q) + adz * dEx;
                el2(pz, q) = on ? p : el2(pz, q);
                vz += el2(pz, q);
              }
              const float dEz = (e < 3 ? el(ez[j], e + 1) : ezn) - el(ez[j], e);
              float vx = dEz * el(ikx4, e);
              if (xs) {
                const float p = el2(bxx, q) * el2(px, q) + el2(adx, q) * dEz;
                el2(px, q) = on ? p : el2(px, q);
                vx += el2(px, q);
              }
              const float h = el(hy[j], e) + dbH * (vx + vz);
              el(hv, e) = on ? h : el(hy[j], e);
            }
            if (zs[j]) sts2(sMExz + so + 2 * hh, pz);
            if (xs) sts2(sMEzx + so + 2 * hh, px);
          }
        }
        hy[j] = hv;
        sHyCol[row * SX + tx + 1] = hv.w;
        if (right && tx == TXT - 1) ll_put1(ecol(par, 1, bx) + k, hv.w, tag);
        if (j == RB - 1) sts4(sHyRow + (ty + 1) * TW + 4 * tx, hv);
        if (down && row == nzt - 1) ll_put4(erow(par, 1, bz) + i0, hv, tag);
      }
    } else if (xwarp) {  // Hy row above and column on the left for this step's E half
      if (!fetch_edges(up ? erow(par, 1, bz - 1) + x0 : nullptr, sHyRow, up ? 4 * nc4 : 0,
                       left ? ecol(par, 1, bx - 1) + z0 : nullptr, sHyCol, SX, left ? nzt : 0, tag + a.tag_bias, ctl,
                       a.limit_ns) &&
          (tid & 31) == 0)
        s_abort = 1;
    }
    __syncthreads();
    if (s_abort) {
      ok = false;
      break;
    }

    // ================= E half-step, source, Dirichlet planes, norm (:273-321)
    if (cell) {
      const float4 hmt = lds4(sHyRow + ty * TW + 4 * tx);
#pragma unroll
      for (int j = 0; j < RB; ++j) {
        if (j >= nrows) continue;
        const int row = rbase + j, k = z0 + row, so = 4 * (j * kResCellThreads + tid);
        float4 hm = hmt;
        if (j > 0) hm = hy[j > 0 ? j - 1 : 0];
        const float hl = sHyCol[row * SX + tx];
        const float4 h = hy[j];
        const float4 cxa = lds4(sCAx + so), cxb = lds4(sCBx + so), cza = lds4(sCAz + so), czb = lds4(sCBz + so);
        if (INTERIOR || fast) {
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const float dHz = el(h, e) - el(hm, e);
            const float exv = el(cxa, e) * el(ex[j], e) + el(cxb, e) * (dHz * ikzh[j]);
            const float dHx = el(h, e) - (e == 0 ? hl : el(h, e - 1));
            const float ezv = el(cza, e) * el(ez[j], e) + el(czb, e) * (dHx * el(ikxh4, e));
            float exs = exv, ezs = ezv;
            if (INTERIOR && hsrc && 4 * j + e == se) {  // :300-301, the source inside an interior tile
              exs += a.io.src[t];
              ezs += a.io.src[a.io.nstep + t];
            }
            el(ex[j], e) = exs;
            el(ez[j], e) = ezs;
            nrm = fmaxf(nrm, norm_monitor(exs, ezs));
          }
        } else if constexpr (!INTERIOR) {  // strip, bound or plane cells: two cells at a time, masks applied as selects
          const unsigned mj = m[j];
          const bool rowplain = (mj & 0xffffffu) == 0x000fffu;
          float adz = 0.0f, bzc = 0.0f;
          if (zs[j]) {
            adz = __ldg(a.Z.adh + k);
            bzc = __ldg(a.Z.bh + k);
          }
#pragma unroll
          for (int hh = 0; hh < 2; ++hh) {
            float2 pz = make_float2(0.f, 0.f), px = pz, adx = pz, bxx = pz;
            if (zs[j]) pz = lds2(sMHyz + so + 2 * hh);
            if (xs) {
              px = lds2(sMHyx + so + 2 * hh);
              adx = ld2(a.X.adh + i0 + 2 * hh);
              bxx = ld2(a.X.bh + i0 + 2 * hh);
            }
#pragma unroll
            for (int q = 0; q < 2; ++q) {
              const int e = 2 * hh + q;
              const bool upx = rowplain || mbit(mj, kMEX, e), upz = rowplain || mbit(mj, kMEZ, e);
              const float dHz = el(h, e) - el(hm, e);
              float d = dHz * ikzh[j];
              if (zs[j]) {
                const float p = bzc * el2(pz, q) + adz * dHz;
                el2(pz, q) = upx ? p : el2(pz, q);
                d += el2(pz, q);
              }
              float exv = el(cxa, e) * el(ex[j], e) + el(cxb, e) * d;
              exv = upx ? exv : el(ex[j], e);
              const float dHx = el(h, e) - (e == 0 ? hl : el(h, e - 1));
              float d2 = dHx * el(ikxh4, e);
              if (xs) {
                const float p = el2(bxx, q) * el2(px, q) + el2(adx, q) * dHx;
                el2(px, q) = upz ? p : el2(px, q);
                d2 += el2(px, q);
              }
              float ezv = el(cza, e) * el(ez[j], e) + el(czb, e) * d2;
              ezv = upz ? ezv : el(ez[j], e);
              if (4 * j + e == se) {  // :300-301
                exv += a.io.src[t];
                ezv += a.io.src[a.io.nstep + t];
              }
              if (!rowplain) {  // :304-312
                if (mbit(mj, kMEXZ, e)) exv = 0.0f;
                if (mbit(mj, kMEZZ, e)) ezv = 0.0f;
              }
              el(ex[j], e) = exv;
              el(ez[j], e) = ezv;
              if (rowplain || mbit(mj, kMCELL, e)) nrm = fmaxf(nrm, norm_monitor(exv, ezv));
            }
            if (zs[j]) sts2(sMHyz + so + 2 * hh, pz);
            if (xs) sts2(sMHyx + so + 2 * hh, px);
          }
        }
        sEzCol[row * SX + tx] = ez[j].x;
        if (left && tx == 0) ll_put1(ecol(par ^ 1, 0, bx) + k, ez[j].x, tag + 1u);
      }
      sts4(sExRow + ty * TW + 4 * tx, ex[0]);
      if (up && rbase == 0) ll_put4(erow(par ^ 1, 0, bz) + i0, ex[0], tag + 1u);
      if (DUMP) {  // the state after step t, each thread its own cells; Hy before its planes are zeroed
        char* d = a.dump.base + (size_t)(s + 1) * a.dump.stride;
#pragma unroll
        for (int j = 0; j < RB; ++j) {
          if (j >= nrows) continue;
          const int row = rbase + j, k = z0 + row;
          const int gg = k * P + i0, so = 4 * (j * kResCellThreads + tid);
          // streaming stores: the copies are read back only after the run
          __stcs(reinterpret_cast<float4*>((float*)(d + a.dump.off[0]) + gg), ex[j]);
          __stcs(reinterpret_cast<float4*>((float*)(d + a.dump.off[1]) + gg), ez[j]);
          __stcs(reinterpret_cast<float4*>((float*)(d + a.dump.off[2]) + gg), hy[j]);
          if (zs[j]) {
            const int zrow = strip_idx(k, NZ, W) * P + i0;
            __stcs(reinterpret_cast<float4*>((float*)(d + a.dump.off[3]) + zrow), lds4(sMExz + so));
            __stcs(reinterpret_cast<float4*>((float*)(d + a.dump.off[5]) + zrow), lds4(sMHyz + so));
          }
          if (xs) {
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const int i = i0 + e;
              if (i < NX && in_strip(i, NX, W)) {
                const int q = k * (2 * W) + strip_idx(i, NX, W);
                ((float*)(d + a.dump.off[4]))[q] = sMEzx[so + e];
                ((float*)(d + a.dump.off[6]))[q] = sMHyx[so + e];
              }
            }
          }
        }
      }
      if (!INTERIOR && !plain) {  // the stored Hy keeps its Dirichlet planes at zero, after every row's E used it
#pragma unroll
        for (int j = 0; j < RB; ++j)
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (mbit(m[j], kMHYZ, e)) el(hy[j], e) = 0.0f;
      }
      if (CKPT && (s + 1) % a.ckpt_every == 0 && s + 1 < a.nsteps) {
        // a checkpoint: the state the handle would hold after step t, in the
        // sfd_checkpoint_save layout (scalar stores: the caller's rows need
        // only 4-byte alignment)
        char* d = a.ckpt.base + (size_t)((s + 1) / a.ckpt_every) * a.ckpt.stride;
#pragma unroll
        for (int j = 0; j < RB; ++j) {
          if (j >= nrows) continue;
          const int row = rbase + j, k = z0 + row;
          const int gg = k * P + i0, so = 4 * (j * kResCellThreads + tid);
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int i = i0 + e;
            if (i >= NX) continue;
            __stcs((float*)(d + a.ckpt.off[0]) + gg + e, el(ex[j], e));
            __stcs((float*)(d + a.ckpt.off[1]) + gg + e, el(ez[j], e));
            __stcs((float*)(d + a.ckpt.off[2]) + gg + e, el(hy[j], e));
            if (zs[j]) {
              const int zrow = strip_idx(k, NZ, W) * P + i;
              __stcs((float*)(d + a.ckpt.off[3]) + zrow, sMExz[so + e]);
              __stcs((float*)(d + a.ckpt.off[5]) + zrow, sMHyz[so + e]);
            }
            if (!INTERIOR && in_strip(i, NX, W)) {
              const int q = k * (2 * W) + strip_idx(i, NX, W);
              __stcs((float*)(d + a.ckpt.off[4]) + q, sMEzx[so + e]);
              __stcs((float*)(d + a.ckpt.off[6]) + q, sMHyx[so + e]);
            }
          }
        }
      }
      if (recm) {  // receivers of step t
        float* tr = a.io.traces + (size_t)t * 2 * a.io.nrec;
#pragma unroll
        for (int j = 0; j < RB; ++j)
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            if (!(recm & (1u << (4 * j + e)))) continue;
            const int c = (rbase + j) * TW + 4 * tx + e;
            if (nloc <= kResMaxLocalRec) {
              for (int q = 0; q < nloc; ++q)
                if (s_rec[2 * q + 1] == c) {
                  tr[s_rec[2 * q]] = el(ex[j], e);
                  tr[a.io.nrec + s_rec[2 * q]] = el(ez[j], e);
                }
            } else {
              for (int q = 0; q < a.io.nrec; ++q)
                if (a.io.rec[3 * q] == i0 + e && a.io.rec[3 * q + 2] == z0 + rbase + j) {
                  tr[q] = el(ex[j], e);
                  tr[a.io.nrec + q] = el(ez[j], e);
                }
            }
          }
      }
    } else if (xwarp && s + 1 < a.nsteps) {  // Ex row below and Ez column to the right for step s+1
      if (!fetch_edges(down ? erow(par ^ 1, 0, bz + 1) + x0 : nullptr, sExRow + TYT * TW, down ? 4 * nc4 : 0,
                       right ? ecol(par ^ 1, 0, bx + 1) + z0 : nullptr, sEzCol + TXT, SX, right ? nzt : 0, tag + 1u + a.tag_bias,
                       ctl, a.limit_ns) &&
          (tid & 31) == 0)
        s_abort = 1;
    }
    __syncthreads();
    if (s_abort) ok = false;
  }
  if (!ok) return;  // the state is left as it was loaded; the host reports the timeout

  // ---- write the cells back (a recompute run for the adjoint keeps its input)
  if (cell && !DUMP) {
#pragma unroll
    for (int j = 0; j < RB; ++j) {
      if (j >= nrows) continue;
      const int row = rbase + j, k = z0 + row;
      const int gg = k * P + i0, so = 4 * (j * kResCellThreads + tid);
      st4(a.Ex + gg, ex[j]);
      st4(a.Ez + gg, ez[j]);
      st4(a.Hy + gg, hy[j]);
      if (zs[j]) {
        const int zrow = strip_idx(k, NZ, W) * P + i0;
        st4(a.mExz + zrow, lds4(sMExz + so));
        st4(a.mHyz + zrow, lds4(sMHyz + so));
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = i0 + e;
        if (!INTERIOR && i < NX && in_strip(i, NX, W)) {
          const int q = k * (2 * W) + strip_idx(i, NX, W);
          a.mEzx[q] = sMEzx[so + e];
          a.mHyx[q] = sMHyx[so + e];
        }
      }
    }
  }
  block_norm_to_slot(nrm, a.io.slots, tile);
}

template <int MODE>
__global__ void __launch_bounds__(kResThreads, 1) em2_resident_kernel(const __grid_constant__ Em2Resident a) {
  extern __shared__ __align__(16) float smem[];
  __shared__ int s_abort, s_nrec;
  __shared__ int s_rec[2 * kResMaxLocalRec];  // (receiver, tile cell) pairs
  if (a.plan.tile[blockIdx.x].w >> 16) em2_resident_tile<MODE, kResRows3>(a, smem, s_abort, s_nrec, s_rec);
  else em2_resident_tile<MODE, kResRows>(a, smem, s_abort, s_nrec, s_rec);
}

}  // namespace

size_t em2_resident_smem(int TW, int TZ, int RB) {
  const size_t SX = (size_t)TW / 4 + 1, TYT = ((size_t)TZ + RB - 1) / RB;
  const size_t arrays = RB == kResRows3 ? 4 : 8;  // coefficients, and the memory variables outside interior tiles
  return sizeof(float) * (4 * arrays * (size_t)RB * kResCellThreads + 2 * (TYT + 1) * TW + 2 * (size_t)TZ * SX);
}

namespace {

// Cost model of the planner, in four-cell groups: a group in a CPML strip or
// on a boundary plane takes the longer update, this many times an interior
// group's.  The forward kernel's weight with interior three-row tiles, and
// the adjoint sweep's (kResRows everywhere); build-time tunables, the
// defaults measured best on the 1040 x 540 grid (forward: 4.26 us per step
// at 6, 4.35 at 4, 4.50 with no three-row tiles, same box).
#ifndef SFD_RES_GENERAL_COST
#define SFD_RES_GENERAL_COST 6.0
#endif
#ifndef SFD_RES_ADJ_GENERAL_COST
#define SFD_RES_ADJ_GENERAL_COST 4.0
#endif

// Cut n items of weight 1 + beta * gen[q] into `parts` runs of about equal
// weight; bounds[0] = 0, bounds[parts] = n.  False if a run would be empty.
bool cut_weighted(int n, const std::vector<int>& gen, double beta, int parts, int* bounds) {
  std::vector<double> acc(n + 1, 0.0);
  for (int q = 0; q < n; ++q) acc[q + 1] = acc[q] + 1.0 + beta * gen[q];
  bounds[0] = 0;
  int q = 0;
  for (int c = 1; c < parts; ++c) {
    const double target = acc[n] * c / parts;
    while (q < n && acc[q] < target) ++q;
    q = std::max(q, bounds[c - 1] + 1);
    if (q > n - (parts - c)) return false;
    bounds[c] = q;
  }
  bounds[parts] = n;
  return true;
}

}  // namespace

bool em2_resident_plan(int NX, int NZ, int npml, int max_ctas, size_t max_smem, ResPlan* out, bool rows3) {
  const int W = npml;
  const double kGeneralCost = rows3 ? SFD_RES_GENERAL_COST : SFD_RES_ADJ_GENERAL_COST;
  const int ng = (NX + 3) / 4;  // four-cell column groups
  std::vector<int> gcol(ng), grow(NZ);
  for (int g = 0; g < ng; ++g) {
    int gen = 4 * g + 3 >= NX ? 1 : 0;
    for (int i = 4 * g; i < std::min(NX, 4 * g + 4); ++i) gen |= (i < W || i >= NX - W || i < 1 || i > NX - 3) ? 1 : 0;
    gcol[g] = gen;
  }
  for (int k = 0; k < NZ; ++k) grow[k] = (k < W || k >= NZ - W || k < 1 || k > NZ - 3) ? 1 : 0;
  std::vector<int> pr(NZ + 1, 0);
  for (int k = 0; k < NZ; ++k) pr[k + 1] = pr[k] + grow[k];
  max_ctas = std::min(max_ctas, kResMaxTiles);

  // Whether a tile of ngp groups and nr rows fits one CTA with RB rows per thread.
  auto fits = [&](int ngp, int nr, int RB) {
    return ngp * ((nr + RB - 1) / RB) <= kResCellThreads && 4 * ngp + nr <= 32 * kResFetchPerLane &&
           em2_resident_smem(4 * ngp, nr, RB) <= max_smem;
  };
  // Cut tile row [z0, z1) into tiles of cost <= C, greedily from the left;
  // returns the tile count (or a count above max_ctas if impossible) and
  // the group bounds in `cuts`, and in `inner` whether each tile is interior
  // (kResRows3 rows per thread).
  auto cut_row = [&](int z0, int z1, double C, std::vector<int>* cuts, std::vector<char>* inner) {
    const int nr = z1 - z0, gr = pr[z1] - pr[z0];
    const bool band3 = rows3 && gr == 0;  // no strip or boundary row in the band
    int count = 0, g0 = 0;
    bool in3 = band3;  // the open tile holds interior groups only
    double cost = 0.0;
    if (cuts) cuts->assign(1, 0);
    if (inner) inner->clear();
    for (int g = 0; g < ng; ++g) {
      const double cg = gcol[g] ? kGeneralCost * nr : gr * kGeneralCost + (nr - gr);
      bool in3g = in3 && !gcol[g];
      const bool over = cost + cg + 1.0 + nr > C || !fits(g - g0 + 1, nr, in3g ? kResRows3 : kResRows);
      if (over && g > g0) {
        ++count;
        if (cuts) cuts->push_back(g);
        if (inner) inner->push_back(in3);
        g0 = g;
        cost = 0.0;
        in3g = band3 && !gcol[g];
      }
      if (!fits(g - g0 + 1, nr, in3g ? kResRows3 : kResRows) || cg + 1.0 + nr > C)
        return max_ctas + 1;  // one group alone does not fit
      in3 = in3g;
      cost += cg + 1.0;
    }
    ++count;
    if (cuts) cuts->push_back(ng);
    if (inner) inner->push_back(in3);
    return count > kResMaxTiles1D ? max_ctas + 1 : count;
  };

  const double betas[] = {0.0, 1.0, 2.0, 3.0, 5.0, 8.0};
  double best = 0.0;
  bool found = false;
  int best_rows[kResMaxTiles1D + 1], best_ntz = 0;
  int rb[kResMaxTiles1D + 1];
  for (int ntz = 1; ntz <= std::min(kResMaxTiles1D, NZ); ++ntz) {
    for (double bzw : betas) {
      if (!cut_weighted(NZ, grow, bzw, ntz, rb)) continue;
      double lo = 0.0, hi = 1e12;
      auto tiles_at = [&](double C) {
        int total = 0;
        for (int r = 0; r < ntz && total <= max_ctas; ++r) total += cut_row(rb[r], rb[r + 1], C, nullptr, nullptr);
        return total;
      };
      if (tiles_at(hi) > max_ctas) continue;
      for (int it = 0; it < 40 && hi - lo > 0.5; ++it) {
        const double mid = 0.5 * (lo + hi);
        (tiles_at(mid) <= max_ctas ? hi : lo) = mid;
      }
      if (!found || hi < best * (1.0 - 1e-9)) {
        best = hi;
        found = true;
        best_ntz = ntz;
        for (int r = 0; r <= ntz; ++r) best_rows[r] = rb[r];
      }
    }
  }
  if (!found) return false;
  out->ntz = best_ntz;
  out->ntiles = 0;
  out->smem = 0;
  std::vector<int> cuts;
  std::vector<char> inner;
  for (int r = 0; r < best_ntz; ++r) {
    const int z0 = best_rows[r], z1 = best_rows[r + 1];
    const int n = cut_row(z0, z1, best, &cuts, &inner);
    for (int c = 0; c < n; ++c) {
      const int x0 = 4 * cuts[c], x1 = std::min(NX, 4 * cuts[c + 1]);
      out->tile[out->ntiles++] = make_int4(x0 | (x1 << 16), z0 | (z1 << 16), r | (c << 16), n | (inner[c] << 16));
      out->smem = std::max(out->smem, em2_resident_smem((x1 - x0 + 3) & ~3, z1 - z0, inner[c] ? kResRows3 : kResRows));
    }
  }
  return true;
}

cudaError_t em2_resident_prepare(const ResPlan& plan, int* ctas_per_sm) {
  const void* fns[3] = {(const void*)em2_resident_kernel<0>, (const void*)em2_resident_kernel<1>,
                        (const void*)em2_resident_kernel<2>};
  int n = 1 << 30;
  for (const void* fn : fns) {
    cudaError_t e = res_allow_max_smem(fn);
    int q = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, fn, kResThreads, plan.smem);
    if (e != cudaSuccess) return e;
    n = std::min(n, q);
  }
  *ctas_per_sm = n;
  return cudaSuccess;
}

cudaError_t em2_resident_launch(const Em2Resident& a, cudaStream_t s) {
  void* args[] = {(void*)&a};
  const void* fn = a.dump.base   ? (const void*)em2_resident_kernel<1>
                   : a.ckpt.base ? (const void*)em2_resident_kernel<2>
                                 : (const void*)em2_resident_kernel<0>;
  return cudaLaunchCooperativeKernel(fn, dim3(a.plan.ntiles), dim3(kResThreads), args, a.plan.smem, s);
}

}  // namespace sfd
