// Host-side argument blocks and launchers of the four solvers.  One struct per
// solver holds the device pointers of a handle; kernels take it by value.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include "sfd_common.cuh"

namespace sfd {

// Receivers + traces + control shared by all solvers.
struct IoArgs {
  Ctl* ctl;
  float* slots;       // one norm slot per block of the second half-step kernel
  const float* src;   // [ncomp][nstep] amplitudes already scaled by dt/rho or dt/eps
  // seismic stress source at the same cell, [ncomp][nstep] amplitudes scaled
  // by dt (xx zz xz in 2-D; xx yy zz xy xz yz in 2.5-D), added to the
  // stresses after the stress half-step; NULL when the handle has none
  const float* ssrc;
  int nstep;
  int si, sj, sk;     // source cell
  const int* rec;     // [nrec][3]
  int nrec;
  float* traces;      // [nstep][nch][nrec]
};

// The driver's 2-D CPML coefficients (SFD_FLAG_CPML_2D): FP32 planes of
// pitch P, [0] of the full offset, [1] of the half offset: 1/K, a, b; and
// 1/dx, 1/dz.  Empty (null planes) otherwise.
struct Cpml2d {
  const float *ik[2], *a[2], *b[2];
  float idx, idz;
};

struct Em2Args {
  int NX, NZ, P, W;
  float *Ex, *Ez, *Hy;
  float *mExz, *mEzx, *mHyz, *mHyx;  // z-, x-, z-, x-strip
  // staggered-averaged update coefficients, (c(i,k) + c(i,k-1))/2 at Ex and
  // (c(i,k) + c(i-1,k))/2 at Ez (electromagfdtd.f95:282, 294), formed in FP64
  const float *CAx, *CBx, *CAz, *CBz;
  AxisTab X, Z;
  float dbH;
  Cpml2d c2d;
  IoArgs io;
};

// electromag2c: complex permittivities (electromagfdtd.f95:329-616).  Every
// complex array is a pair of planes, [0] real and [1] imaginary.
struct Em2cArgs {
  int NX, NZ, P, W;
  float *Ex[2], *Ez[2], *Hy[2];
  float *mExz[2], *mEzx[2], *mHyz[2], *mHyx[2];  // z-, x-, z-, x-strip
  const float *CAx[2], *CBx[2], *CAz[2], *CBz[2];  // staggered averages of the complex coefficients
  AxisTab X, Z;
  float dbH;
  IoArgs io;  // source rows and trace channels: Ex re, Ex im, Ez re, Ez im
};

struct Seis2Args {
  int NX, NZ, P, W;
  int atten;
  int legacy;  // 1: the legacy loops' quirks (shared memory variables, b_x_half(j)); 0: corrected physics
  float *vx, *vz, *sxx, *szz, *sxz;
  float *m_vxx, *m_vzz, *m_vxz, *m_vzx;      // x, z, z, x strips
  float *m2_vxx, *m2_vzz, *m2_vxz, *m2_vzx;  // the sigmaxz loop's own (corrected physics), same strips
  float *m_sxx_x, *m_szz_z, *m_sxz_x, *m_sxz_z;  // x, z, x, z strips
  // dt * averaged stiffness, formed in FP64: (c(i+1,j) + 2c(i,j) + c(i,j-1))/4
  // at the normal-stress points (seismicfdtd.f95:270-280) and
  // (c(i,j+1) + 2c(i,j) + c(i-1,j))/4 at the shear-stress points (:306-311)
  const float *A11, *A13, *A15, *A33, *A35, *B15, *B35, *B55;
  const float *dtrx, *dtrz;                      // dt / rho, dt / rho_avg
  const float *gxp, *gzp;                        // 1 - gamma
  const float* q3;                               // b_x_half indexed by the z index (legacy loop 1)
  AxisTab X, Z;
  Cpml2d c2d;
  IoArgs io;
};

struct Seis25Args {
  int NX, NY, NZ, P, W;
  int atten;
  int legacy;  // 1: the legacy coefficient pairs of c16 and c45 (seismicfdtd.f95:657, 766); 0: Voigt pairs
  float *vx, *vy, *vz, *sxx, *syy, *szz, *sxy, *sxz, *syz;
  // velocity-gradient memory (shared by the four stress loops)
  float *m_vx_x, *m_vy_x, *m_vz_x;  // x-strip
  float *m_vx_y, *m_vy_y, *m_vz_y;  // y-strip
  float *m_vx_z, *m_vy_z, *m_vz_z;  // z-strip
  // stress-gradient memory
  float *m_sxx_x, *m_sxy_x, *m_sxz_x;  // x-strip
  float *m_syy_y, *m_sxy_y, *m_syz_y;  // y-strip
  float *m_szz_z, *m_sxz_z, *m_syz_z;  // z-strip
  const float* C;     // 33 planes: the stress loops' stiffness averages x dt, pitch P, NZ rows each
  const float* dtr;   // 3 planes: dt / rho_avg for vx, vy, vz
  const float* gp;    // 3 planes: 1 - gamma_x, 1 - gamma_y, 1 - gamma_z
  AxisTab X, Y, Z;
  float idx, idz;     // 1/dx, 1/dz for the derivatives :701-707 leaves unscaled
  int ysplit;         // y segments per column (work split of the y march)
  IoArgs io;
  // TMA descriptors of the nine fields as one (NX, NY, NZ, 9) FP32 tensor
  // (seis25_make_maps): velocities with a halo and the stresses of the own
  // cells (stress kernel), stresses with a halo and the velocities of the own
  // cells (velocity kernel)
  CUtensorMap tm_vhalo, tm_sown, tm_shalo, tm_vown;
  // the y-strip memory variables of each kernel (three arrays, equally
  // spaced) and the y axis table, staged with the planes
  CUtensorMap tm_ypsi_v, tm_ypsi_s, tm_ytab;
  unsigned long long wait_ns;  // bound of each wait for a staged tile
  unsigned stall_tx;           // test aid: extra bytes each stage expects (0; > 0 makes the waits run out)
};

struct Em25Args {
  int NX, NY, NZ, P, W;
  float *Ex, *Ey, *Ez, *Hx, *Hy, *Hz;
  float *mEz_y, *mEy_z, *mEx_z, *mEz_x, *mEx_y, *mEy_x;
  float *mHz_y, *mHy_z, *mHz_x, *mHx_z, *mHx_y, *mHy_x;
  const float *caEx, *cbEx, *caEy, *cbEy, *caEz, *cbEz;
  AxisTab X, Y, Z;
  float dbH;
  int ysplit;
  IoArgs io;
  // TMA descriptors of the six fields as one (NX, NY, NZ, 6) FP32 tensor
  // (em25_make_maps): three fields with a halo, three of the own cells
  CUtensorMap tm_halo, tm_own;
  // the y-strip memory variables each kernel reads (dEz_dy dEx_dy; dHz_dy
  // dHx_dy) and the y axis table, staged with the planes
  CUtensorMap tm_ypsi_e, tm_ypsi_h, tm_ytab;
  unsigned long long wait_ns;  // bound of each wait for a staged tile
  unsigned stall_tx;           // test aid: extra bytes each stage expects (0; > 0 makes the waits run out)
};

// Single-pass (fused) 2-D steps.  Each launch reads the "old" copy of every
// field and of the memory variables that neighbouring tiles re-derive, and
// writes the "new" copy; memory variables touched only by their owner cell
// are updated in place.  A tile of TX x (8*ZB) cells recomputes the first
// half-step on a one-cell halo so the second half-step needs no second pass.
struct Em2Step {
  int NX, NZ, P, W;
  const float *Ex0, *Ez0, *Hy0, *mExz0, *mEzx0;  // old
  float *Ex1, *Ez1, *Hy1, *mExz1, *mEzx1;        // new
  const float *mHyz0, *mHyx0;                    // second-half memory, read ...
  float *mHyz, *mHyx;                            // ... and written (the same arrays except in adjoint recompute)
  const float *CAx, *CBx, *CAz, *CBz;  // staggered averages, as in Em2Args
  AxisTab X, Z;
  float dbH;
  IoArgs io;
};

struct Seis2Step {
  int NX, NZ, P, W;
  int atten;
  int legacy;  // as Seis2Args
  const float *vx0, *vz0, *sxx0, *szz0, *sxz0;
  float *vx1, *vz1, *sxx1, *szz1, *sxz1;
  const float *m_vxx0, *m_vzz0, *m_vxz0, *m_vzx0;  // velocity-gradient memory, old
  float *m_vxx1, *m_vzz1, *m_vxz1, *m_vzx1;        // new
  const float *m2_vxx0, *m2_vzz0, *m2_vxz0, *m2_vzx0;  // the sigmaxz loop's own (corrected physics), old
  float *m2_vxx1, *m2_vzz1, *m2_vxz1, *m2_vzx1;        // new
  float *m_sxx_x, *m_szz_z, *m_sxz_x, *m_sxz_z;    // in place
  const float *A11, *A13, *A15, *A33, *A35, *B15, *B35, *B55, *dtrx, *dtrz, *gxp, *gzp, *q3;
  AxisTab X, Z;
  IoArgs io;
};

// A material table passed by value to the coefficient kernels of
// sfd_set_model_ids: nmat rows of the kind's model planes, FP64.
constexpr int kMatTableMax = 2048;
struct MatTable {
  int nmat;
  double v[kMatTableMax];
};
// FP32 coefficient planes (plane stride `plane`, row pitch P) of an
// electromag2 or seismic2 handle from a device material-id map; *bad is set
// to 1 if an id is outside [0, nmat).
void coef_from_ids(int kind, const int* ids, const MatTable& m, int NX, int NZ, int P, double dt, float* coef,
                   size_t plane, int* bad, int flags, cudaStream_t s);

// Launch geometry of a solver's two half-step kernels.
struct Launch {
  dim3 grid, block;
  int nslots;
};

Launch em2c_launch(const Em2cArgs& a);
void em2c_half1(const Em2cArgs& a, const Launch& L, int rel, cudaStream_t s);
void em2c_half2(const Em2cArgs& a, const Launch& L, int rel, cudaStream_t s);
void em2c_finalize(const Em2cArgs& a, int t_last, cudaStream_t s);
Launch em2_launch(const Em2Args& a);
void em2_half1(const Em2Args& a, const Launch& L, int rel, cudaStream_t s);
void em2_half2(const Em2Args& a, const Launch& L, int rel, cudaStream_t s);
void em2_finalize(const Em2Args& a, int t_last, cudaStream_t s);

// Two-pass steps with the driver's 2-D CPML fields (cpml2d.cu).
void em2_c2d_half1(const Em2Args& a, const Launch& L, int rel, cudaStream_t s);
void em2_c2d_half2(const Em2Args& a, const Launch& L, int rel, cudaStream_t s);
void seis2_c2d_half1(const Seis2Args& a, const Launch& L, int rel, cudaStream_t s);
void seis2_c2d_half2(const Seis2Args& a, const Launch& L, int rel, cudaStream_t s);

Launch seis2_launch(const Seis2Args& a);
void seis2_half1(const Seis2Args& a, const Launch& L, int rel, cudaStream_t s);
void seis2_half2(const Seis2Args& a, const Launch& L, int rel, cudaStream_t s);
void seis2_finalize(const Seis2Args& a, int t_last, cudaStream_t s);

// Encodes a's four tensor maps over its field array (fields contiguous,
// `field_stride` floats apart); false when the driver refuses one.
bool seis25_make_maps(Seis25Args& a, size_t field_stride, const float* ytab);
Launch seis25_launch(const Seis25Args& a);
void seis25_half1(const Seis25Args& a, const Launch& L, int rel, cudaStream_t s);
void seis25_half2(const Seis25Args& a, const Launch& L, int rel, cudaStream_t s);
void seis25_finalize(const Seis25Args& a, int t_last, cudaStream_t s);

// A 4-D (x, y, z, field) FP32 tensor map over `nfields` fields of (NX, NY,
// NZ) cells at `base` (row pitch P floats, fields `field_stride` floats
// apart) with boxes of box_x x 1 x box_z x box_f (tma_maps.cu).
bool encode_field_map(CUtensorMap* map, void* base, int NX, int NY, int NZ, int P, size_t field_stride, int nfields,
                      int box_x, int box_z, int box_f);
// Any FP32 tiled map: rank dims (innermost first), rank - 1 byte strides.
bool encode_tiled(CUtensorMap* map, void* base, int rank, const cuuint64_t* dims, const cuuint64_t* strides,
                  const cuuint32_t* box);
bool em25_make_maps(Em25Args& a, size_t field_stride, const float* ytab);
Launch em25_launch(const Em25Args& a);
void em25_half1(const Em25Args& a, const Launch& L, int rel, cudaStream_t s);
void em25_half2(const Em25Args& a, const Launch& L, int rel, cudaStream_t s);
void em25_finalize(const Em25Args& a, int t_last, cudaStream_t s);

}  // namespace sfd

struct sfd_config;
struct sfd_handle_s;

namespace sfd {

int32_t create_handle(const sfd_config* cfg, void* dev_state, size_t state_bytes, void* stream, bool graphs,
                      sfd_handle_s** out);
void set_error(const char* msg);

// Fused steps (one launch per time step); zb = rows per thread (1, 2 or 4).
Launch em2_step_launch(const Em2Step& a, int zb);
void em2_step(const Em2Step& a, const Launch& L, int zb, int rel, cudaStream_t s);
void em2_step_finalize(const Em2Step& a, int t_last, cudaStream_t s);
Launch seis2_step_launch(const Seis2Step& a, int zb);
void seis2_step(const Seis2Step& a, const Launch& L, int zb, int rel, cudaStream_t s);
void seis2_step_finalize(const Seis2Step& a, int t_last, cudaStream_t s);

// Input assembly on the device (inputs.cu).  A source time function: one
// FP32 row of nstep values per component q, comp[q] * amp * the peak-
// normalised wavelet, times dt, over div[q].
struct WaveletComp {
  int n;
  double comp[6];
  double div[6];
};
cudaError_t wavelet_launch(int stype, double f0, double dt, int nstep, double amp, const WaveletComp& wc, float* out,
                           size_t stride, cudaStream_t s);
// One axis of CPML profiles into its FP32 table (6 rows of st floats).
struct CpmlAxisArgs {
  int n, npml;
  double delta, dt, sig_max, alpha_max, kappa_max, NP, NPA;
  int seismic, legacy;
};
cudaError_t cpml_axis_launch(const CpmlAxisArgs& p, float* tab, int st, cudaStream_t s);
cudaError_t cpml_q3_launch(const float* bxh, int nx, int nz, float* q3, cudaStream_t s);

// Block-floating int16 encoding of one field (snapshot.cu): minmax[0..1] <-
// the field's min and max, out <- the dense x-fastest int16 codes.  rows =
// NY * NZ rows of NX values at pitch P.  Queued on stream s.
void encode_field_i16(const float* field, int NX, int P, long rows, short* out, float* minmax, cudaStream_t s);

}  // namespace sfd
