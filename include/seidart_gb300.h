/*
 * seidart_gb300 -- C ABI of the GB300 FDTD time-stepping backend.
 *
 * Drop-in for the in-process solver boundary of SeidarT: the f2py-exposed
 * Fortran subroutines
 *   seismic2(nx, nz, dx, dz, npoints_pml, src, nstep, OUTPUT_SINGLE)
 *       legacy/fortran/seismicfdtd.f95:12
 *   seismic25(nx, ny, nz, dx, dy, dz, npoints_pml, src, nstep, OUTPUT_SINGLE)
 *       legacy/fortran/seismicfdtd.f95:388
 *   electromag2(nx, nz, dx, dz, npoints_pml, src, nstep, OUTPUT_SINGLE)
 *       legacy/fortran/electromagfdtd.f95:10
 *   electromag25(nx, ny, nz, dx, dy, dz, npoints_pml, src, nstep, OUTPUT_SINGLE)
 *       legacy/fortran/electromagfdtd.f95:619
 * called from legacy/prjrun_101424.py:691-808, and of the `seidartfdtd`
 * process the current driver launches (src/seidart/routines/classes.py:907-924).
 * Where the Fortran reads its inputs from .dat files in the working directory
 * (material_rw / loadcpml / loadsource, legacy/fortran/readwrite_routines.f95:9-37,
 * 451-470) this library takes the same arrays as host pointers; where it writes
 * one snapshot file per step (write_image2/3, readwrite_routines.f95:473-527)
 * this library records receiver traces on the device and exposes every field.
 *
 * Conventions
 *   - All sizes are FULL-grid sizes (CPML included), the nx/ny/nz the Fortran
 *     receives.  Arrays on the host are x fastest (Fortran order): 2-D index
 *     i + NX*k, 2.5-D index i + NX*(j + NY*k).  Indices are 0-based: the
 *     Fortran cell (i, k) is (i-1, k-1) here.
 *   - Material arrays are FP64 (NX, NZ) planes; in 2.5-D they are y-invariant,
 *     as in the Fortran (seismicfdtd.f95:399-405, electromagfdtd.f95:633-638).
 *   - Fields are computed in FP32 on the GPU.  dt, the CPML profiles and the
 *     derived update coefficients are computed in FP64 on the host (the
 *     profiles and the source time functions optionally in FP64 on the device:
 *     sfd_set_cpml_params, sfd_set_source_wavelet).
 *   - The library never allocates device memory: the caller passes one device
 *     buffer of sfd_state_bytes() bytes that holds every field, CPML memory
 *     variable, coefficient, source and trace of the handle.
 *   - Every call returns SFD_OK (0) or a negative SFD_ERR_* code and sets a
 *     thread-local message readable with sfd_last_error().  No call exits or
 *     traps.
 *   - One handle is bound to one CUDA stream; calls on a handle must be
 *     serialised by the caller; different handles are independent.
 */
#ifndef SEIDART_GB300_H
#define SEIDART_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Solver kinds: the Fortran subroutine each one replaces. */
#define SFD_SEISMIC2 1     /* seismicfdtd.f95:12-385    */
#define SFD_SEISMIC25 2    /* seismicfdtd.f95:388-949   */
#define SFD_ELECTROMAG2 3  /* electromagfdtd.f95:10-326 */
#define SFD_ELECTROMAG25 4 /* electromagfdtd.f95:619-1092 */
#define SFD_ELECTROMAG2C 5 /* electromagfdtd.f95:329-616: electromag2 with complex permittivities */

/* Return codes. */
#define SFD_OK 0
#define SFD_ERR_BAD_ARG -1
#define SFD_ERR_STATE -2    /* call out of order (e.g. run before set_model) */
#define SFD_ERR_CUDA -3
#define SFD_ERR_UNSTABLE -4 /* field norm above 1e25 or NaN (seismicfdtd.f95:378-379) */
#define SFD_ERR_TIMEOUT -5  /* a bounded device wait gave up */

/* Flags (sfd_config.flags). */
#define SFD_FLAG_TWO_PASS 1 /* 2-D kinds: two kernels per step (one per half-step,
                               fields updated in place) instead of the default
                               single-pass step over ping-pong copies */
#define SFD_FLAG_STREAMING 2 /* 2-D single-pass kinds: one launch per step even
                               when the grid fits on chip (by default a run of
                               a grid that fits in the SMs' shared memory is
                               one launch with the state held on chip) */
/* Seismic kinds: reproduce the legacy Fortran loops' quirks instead of the
 * default corrected physics.
 *   seismic2: the two stress loops share their four velocity-gradient CPML
 *     memory variables, which so advance twice per step where both loops
 *     visit a cell (seismicfdtd.f95:255-262, 291-298); loop 1 reads
 *     b_x_half at the z index (:255); vx divides by the cell's own rho (:334)
 *     although :320 forms the averaged density.  Corrected: the sigmaxz loop
 *     keeps its own four memory variables, b_x_half(i), and vx divides by
 *     the average of :320.
 *   seismic25: the coefficient pairs c16 (dvx_dy + dvz_dy) (:657) and
 *     c45 (dvx_dz + dvz_dx) (:766).  Corrected: the Voigt pairs c16 (dvx_dy +
 *     dvy_dx) and c45 (dvy_dz + dvz_dy). */
#define SFD_FLAG_LEGACY_QUIRKS 4
/* Seismic kinds: averaging of the density at the staggered velocity points
 * (the driver's density_method argument, src/seidart/routines/classes.py:311,
 * 910-924), a two-bit field.  0 (no flag) = arithmetic, the Fortran's
 * averages (seismicfdtd.f95:320, 342, 825, 850, 876); NONE = the cell's own
 * density; GEOMETRIC and HARMONIC = the weighted geometric and harmonic means
 * over the same stencil (weights 2,1,1 in 2-D, 4,1,1 in 2.5-D). */
#define SFD_FLAG_DENSITY_NONE 8
#define SFD_FLAG_DENSITY_GEOMETRIC 16
#define SFD_FLAG_DENSITY_HARMONIC 24
#define SFD_FLAG_DENSITY_MASK 24
/* electromag2 and seismic2: CPML coefficients from the driver's 2-D fields
 * (sfd_set_cpml2d) instead of per-axis profiles (sfd_set_cpml): every
 * derivative direction takes the field's value at the cell.  The run uses
 * two kernels per step with every CPML memory variable on the full grid;
 * not with SFD_FLAG_LEGACY_QUIRKS (whose loops read 1-D profiles). */
#define SFD_FLAG_CPML_2D 32


typedef struct sfd_config {
  int32_t kind;        /* SFD_SEISMIC2 ... SFD_ELECTROMAG25 */
  int32_t nx, ny, nz;  /* full grid incl. CPML; ny = 1 for 2-D */
  int32_t npml;        /* CPML thickness in cells (npoints_pml) */
  int32_t nstep;       /* length of the source time functions = max steps */
  int32_t nrec;        /* receivers recorded every step */
  int32_t flags;       /* SFD_FLAG_* */
  double dx, dy, dz;   /* grid steps (m); dy ignored in 2-D */
  double dt;           /* time step (s), computed by the caller in FP64 */
} sfd_config;

typedef struct sfd_handle_s sfd_handle;

/* Library version (major*10000 + minor*100 + patch). */
int32_t sfd_version(void);

/* Message of the last failing call on this thread ("" if none). */
const char* sfd_last_error(void);

/* Number of material planes sfd_set_model expects for a kind:
 *   SEISMIC2     9: c11 c13 c15 c33 c35 c55 rho gamma_x gamma_z
 *                   (seismicfdtd.f95:147-159)
 *   SEISMIC25   25: c11 c12 c13 c14 c15 c16 c22 c23 c24 c25 c26 c33 c34 c35
 *                   c36 c44 c45 c46 c55 c56 c66 rho gamma_x gamma_y gamma_z
 *                   (seismicfdtd.f95:476-497; the legacy routine has no
 *                   attenuation: gamma = 0 reproduces it, nonzero gamma applies
 *                   v <- v (1 - gamma) + ... as seismic2 does at :334, 355)
 *   ELECTROMAG2  6: eps11 eps13 eps33 sig11 sig13 sig33
 *                   (electromagfdtd.f95:146-151)
 *   ELECTROMAG25 12: eps11 eps12 eps13 eps22 eps23 eps33
 *                    sig11 sig12 sig13 sig22 sig23 sig33
 *                    (electromagfdtd.f95:729-740)
 *   ELECTROMAG2C  9: eps11 re, im, eps13 re, im, eps33 re, im, sig11 sig13
 *                    sig33 (complex eps read by material_rwc,
 *                    readwrite_routines.f95:969-988; :424-429) */
int32_t sfd_model_planes(int32_t kind);

/* Number of fields and receiver channels of a kind.
 *   SEISMIC2:     vx vz sigmaxx sigmazz sigmaxz                 channels vx vz
 *   SEISMIC25:    vx vy vz sigmaxx sigmayy sigmazz sigmaxy sigmaxz sigmayz
 *                                                               channels vx vy vz
 *   ELECTROMAG2:  Ex Ez Hy                                      channels Ex Ez
 *   ELECTROMAG25: Ex Ey Ez Hx Hy Hz                             channels Ex Ey Ez
 *   ELECTROMAG2C: Ex re, im, Ez re, im, Hy re, im  channels Ex re, Ex im, Ez re, Ez im
 *                 (memory variables likewise in real/imaginary pairs) */
int32_t sfd_num_fields(int32_t kind);
int32_t sfd_num_channels(int32_t kind);
/* Number of CPML memory variables (the Fortran memory_* arrays).  SEISMIC2
 * has 12: dvx_dx dvz_dz dvx_dz dvz_dx dsigmaxx_dx dsigmazz_dz dsigmaxz_dx
 * dsigmaxz_dz, then the sigmaxz loop's own dvx_dx dvz_dz dvx_dz dvz_dx
 * (corrected physics; zero with SFD_FLAG_LEGACY_QUIRKS). */
int32_t sfd_num_memory(int32_t kind);

/* Bytes of device memory a handle of this configuration needs. */
int32_t sfd_state_bytes(const sfd_config* cfg, size_t* bytes);

/* Create a handle over a caller-owned device buffer (>= sfd_state_bytes,
 * 256-byte aligned).  `stream` is a cudaStream_t (NULL = legacy default
 * stream).  Fields, memory variables and traces start at zero. */
int32_t sfd_create(const sfd_config* cfg, void* dev_state, size_t state_bytes, void* stream,
                   sfd_handle** out);

/* Material planes, host FP64, sfd_model_planes(kind) planes of NX*NZ values
 * (count = planes*NX*NZ).  Replaces the material_rw reads of the Fortran. */
int32_t sfd_set_model(sfd_handle* h, const double* planes, int64_t count);

/* The same model as a material-id map: ids, device int32 [NZ][NX] (x
 * fastest, the project image's material index per cell, CPML cells
 * included), values in [0, nmat); table, host FP64 [nmat][planes] in
 * sfd_set_model's plane order (count = nmat * planes, at most 2048 values).
 * The update coefficients are formed on the device, in FP64, with the
 * formulas of sfd_set_model, so both calls store the same coefficients; the
 * FP64 planes never cross to the GPU.  All kinds but electromag2c; for the
 * 2.5-D kinds the map is the (x, z) image of the y-invariant model.  The
 * id map must stay allocated while the handle may set a source or take an
 * adjoint gradient (both read it).  Replaces the driver's expansion of the
 * material table into per-cell .dat files (src/seidart/routines/
 * classes.py:608-750) and their reads (readwrite_routines.f95:9-37). */
int32_t sfd_set_model_ids(sfd_handle* h, const int32_t* ids, int32_t nmat, const double* table, int64_t count);

/* CPML profiles, host FP64: for each axis (x, [y,] z) the arrays
 * K, a, b, K_half, a_half, b_half of the axis length, concatenated
 * (count = 6*(NX + [NY +] NZ)).  Replaces the loadcpml reads
 * (seismicfdtd.f95:202-220).  a and a_half must vanish outside the npml-cell
 * strips at both ends of each axis. */
int32_t sfd_set_cpml(sfd_handle* h, const double* profiles, int64_t count);

/* SFD_FLAG_CPML_2D handles: the driver's 2-D CPML fields, host FP64, six
 * planes of NX*NZ values (x fastest): K, a, b, K_half, a_half, b_half
 * (count = 6*NX*NZ) -- the kappa, acoef, bcoef{,_half}_cpml.dat files the
 * current driver writes (src/seidart/routines/definitions.py:560-998; their
 * records hold the (NX, NZ) arrays x fastest).  The full-offset field is
 * used where the Fortran loops read a full-offset profile, the half-offset
 * field where they read a half-offset one.  K must be positive. */
int32_t sfd_set_cpml2d(sfd_handle* h, const double* fields, int64_t count);

/* Point source at full-grid cell (i, j, k) (j = 0 in 2-D) with time
 * functions srcfn, host FP64, ncomp x nstep values, component-major
 * (x, z in 2-D; x, y, z in 2.5-D).  The value added at step t is
 * srcfn[c][t] * dt / rho (seismic) or * dt / eps_ii (EM), as in
 * seismicfdtd.f95:360-361 and electromagfdtd.f95:300-301.  ELECTROMAG2C
 * takes 2 real components (x, z) divided by the complex eps11, eps33
 * (:581-582).  Requires the model. */
int32_t sfd_set_source(sfd_handle* h, int32_t i, int32_t j, int32_t k, const double* srcfn,
                       int32_t ncomp, int32_t nstep);

/* Seismic kinds: a moment-tensor (stress) source at full-grid cell (i, j, k),
 * the same cell as the force source when both are set.  srcfn, host FP64,
 * ncomp x nstep values, component-major: sigma xx, zz, xz in 2-D (ncomp 3);
 * xx, yy, zz, xy, xz, yz in 2.5-D (ncomp 6).  After the stress half-step of
 * step t, sigma_ij(i, j, k) += srcfn[ij][t] * dt; an explosive source is equal
 * normal components and zero shear.  ncomp = 0 removes the stress source.
 * Replaces the seismicsource{xx,yy,zz,xy,xz,yz}.dat files the driver writes
 * (src/seidart/routines/sourcefunction.py:354-372), which the legacy Fortran
 * never reads. */
int32_t sfd_set_stress_source(sfd_handle* h, int32_t i, int32_t j, int32_t k, const double* srcfn, int32_t ncomp,
                              int32_t nstep);

/* Make dst read src's update coefficients instead of its own (no copy): the
 * shots of one survey share one model.  Same kind, grid, dt and flags
 * (electromag2 or seismic2).  src must outlive dst; a later sfd_set_model on
 * src changes both, one on dst detaches nothing (call it on src).  In a batch,
 * consecutive handles sharing a model run their tiles back to back so the
 * shared coefficients are read from HBM once per step.  Replaces the copy of
 * the model files each shot of the driver's survey loop reads
 * (src/seidart/simulations/common_offset.py:143-176). */
int32_t sfd_share_model(sfd_handle* dst, const sfd_handle* src);

/* ---- Input assembly on the device ------------------------------------------
 * The source time functions and the CPML profiles formed on the GPU in FP64
 * (then stored in FP32 as sfd_set_source / sfd_set_cpml store them), so a
 * caller that loops over models or shots passes a few parameters instead of
 * the arrays.  Replaces the driver's host-side wavelet and cpml_parameters
 * (src/seidart/routines/sourcefunction.py:25-57, 239-300;
 * definitions.py:862-998) and the .dat round trips of their results. */
#define SFD_WAVELET_GAUS0 0 /* Gaussian, width 0.2 / (pi f0) */
#define SFD_WAVELET_GAUS1 1 /* Ricker */
#define SFD_WAVELET_GAUS2 2 /* the driver's 'gaus2' form */
/* The source (stress = 0, as sfd_set_source) or the stress source (stress =
 * 1, as sfd_set_stress_source) at (i, j, k): component c at step t is
 * comp[c] * amp * w(t dt) / max_t |w(t dt)|, w the driver's wavelet of type
 * stype and centre frequency f0 (sourcefunction.py:25-57 on the time vector
 * arange(nstep) * dt, :262; comp the rotation or moment-tensor factors of
 * :276-300).  ncomp as for sfd_set_source / sfd_set_stress_source; not for
 * ELECTROMAG2C. */
int32_t sfd_set_source_wavelet(sfd_handle* h, int32_t stress, int32_t i, int32_t j, int32_t k, int32_t stype,
                               double f0, double amp, const double* comp, int32_t ncomp);

/* CPML profile parameters: per axis (x, [y,] z) the largest conductivity
 * sig_max (seidart_gb300.cpml.sigma_alpha_max gives the driver's and the
 * legacy writer's), and for all axes alpha_max, kappa_max and the exponents
 * NP, NPA; mode 0 = the driver's profiles (distance rescaled to 1 at the
 * outer cell, interior b = 1), 1 = the legacy writer's (interior b = 0). */
typedef struct sfd_cpml_params {
  double sig_max[3];
  double alpha_max;
  double kappa_max;
  double NP, NPA;
  int32_t mode;
} sfd_cpml_params;
/* The profiles of sfd_set_cpml computed on the device from the parameters
 * (seidart_gb300/cpml.py's axis_profile on every axis). */
int32_t sfd_set_cpml_params(sfd_handle* h, const sfd_cpml_params* p);

/* Receiver cells, host int32 (i, j, k) triples, nrec = cfg.nrec. */
int32_t sfd_set_receivers(sfd_handle* h, const int32_t* ijk, int32_t nrec);

/* Zero every field, memory variable and trace and rewind to step 0. */
int32_t sfd_reset(sfd_handle* h);

/* Copy one field between the device state and a host FP32 array of the full
 * grid (count = NX*NY*NZ).  Writing sets initial conditions (the
 * initialcondition*.dat files of classes.py:882-898).  Reads synchronise. */
int32_t sfd_set_field(sfd_handle* h, int32_t field, const float* host, int64_t count);
int32_t sfd_get_field(sfd_handle* h, int32_t field, float* host, int64_t count);
/* The read of sfd_get_field queued on the handle's stream without waiting:
 * `host` may be read once the stream has passed this point (an event
 * recorded after the call, or sfd_status).  Into page-locked host memory
 * the copy overlaps the host's own work; it replaces the per-step snapshot
 * writes of write_image2/write_image3 (readwrite_routines.f95:473-527,
 * called each step at seismicfdtd.f95:381-382 and electromagfdtd.f95:323),
 * whose file output the caller does on its own thread. */
int32_t sfd_get_field_async(sfd_handle* h, int32_t field, float* host, int64_t count);
/* One field as block-floating int16, queued on the handle's stream: device
 * dev_minmax[0..1] <- the field's min and max (FP32), device dev_out (NX*NY*NZ
 * int16, x fastest, then y, then z) <- codes with (code + 32767) / 65534 =
 * (value - min) / (max - min), 0 when max == min.  These are the records of
 * the SEIDART_EM25B1 block files the reference reads for 2.5-D EM snapshots
 * (src/seidart/routines/definitions.py:140-212, read_block); the reference
 * writes them from its Fortran backend, which is not part of its source. */
int32_t sfd_encode_field_i16(sfd_handle* h, int32_t field, void* dev_out, void* dev_minmax);
/* One CPML memory variable expanded to the full grid (zero off its strips). */
int32_t sfd_get_memory(sfd_handle* h, int32_t index, float* host, int64_t count);

/* Advance nsteps time steps (asynchronous on the handle's stream).  The
 * source and the trace index follow the handle's step counter. */
int32_t sfd_run(sfd_handle* h, int64_t nsteps);

/* Synchronise and report: steps done and the largest field norm seen by the
 * last sfd_run.  Returns SFD_ERR_UNSTABLE when that norm exceeded 1e25 or was
 * NaN (the Fortran stops at seismicfdtd.f95:378-379; here the run completes
 * and the status reports it), SFD_ERR_TIMEOUT when an on-chip run gave up
 * waiting for a neighbouring tile (the state is then that before the run). */
int32_t sfd_status(sfd_handle* h, int64_t* step, double* maxnorm);

/* Receiver traces [step][channel][receiver], FP32: copy to host
 * (count = nstep*nchan*nrec) or the device pointer. */
int32_t sfd_get_traces(sfd_handle* h, float* host, int64_t count);
const float* sfd_traces_device(const sfd_handle* h);
/* Device address of field `field` of the handle's current state and its row
 * pitch in floats (x fastest; row (k) of a 2-D field, row (k, j) of a 2.5-D
 * field at ptr + (k*NY + j) * pitch; the NX cells of a row are valid, the
 * rest of the pitch is padding).  For a zero-copy view; single-pass 2-D
 * handles swap between two copies, so the address holds until the next
 * sfd_run, sfd_reset or sfd_checkpoint_load. */
int32_t sfd_field_device(const sfd_handle* h, int32_t field, float** ptr, int64_t* pitch);

/* Profiling aid: launch half-step kernel `which` (0 = first half-step of the
 * Fortran time loop: H or stress; 1 = second: E or velocity) `count` times
 * back to back on the handle's stream without the other half.  Single-pass
 * handles launch their whole-step kernel.  The fields are no longer a valid
 * simulation afterwards; call sfd_reset before the next run. */
int32_t sfd_launch_half(sfd_handle* h, int32_t which, int32_t count);

/* Whether sfd_run keeps this handle's whole state on chip (one launch per run,
 * one CTA per tile of the grid): 1 yes, 0 no (one launch per step).  Single-
 * pass electromag2 and seismic2 handles whose grid fits the SMs' shared
 * memory (and registers) run on chip; decided on the current device from its
 * SM count and shared memory.  tiles and
 * tile_rows (may be NULL) receive the number of tiles and of tile rows.  No
 * counterpart in the reference: its time loop has one execution form. */
int32_t sfd_on_chip(sfd_handle* h, int32_t* tiles, int32_t* tile_rows);

/* Longest wait, in ns, of this handle's on-chip runs (sfd_run, and the
 * adjoint's on-chip recompute and sweep) for a neighbouring tile's edge
 * values; 0 restores the default, 2 s.  A wait that runs out makes every
 * tile leave the run and sfd_status (sfd_adjoint_gradient) return
 * SFD_ERR_TIMEOUT; the context stays usable and sfd_reset starts over.  A
 * correct run never waits near the default: a short limit is how a caller
 * (or a test) checks the timeout path.  No counterpart in the reference. */
int32_t sfd_set_wait_limit(sfd_handle* h, int64_t ns);
/* Test aid for that timeout path: with `on` != 0, the on-chip runs of this
 * handle await edge values under tags no tile ever writes, so every wait runs
 * out after the limit and the run ends with SFD_ERR_TIMEOUT (a flag that
 * nothing sets; no fault, no unbounded wait).  0 restores normal runs. */
int32_t sfd_test_stall_waits(sfd_handle* h, int32_t on);

/* Release the handle (the caller frees its device buffer afterwards). */
int32_t sfd_destroy(sfd_handle* h);

/* ---- One shot without device allocation --------------------------------------
 * For callers that cannot call cudaMalloc (a host application that owns every
 * device allocation and exposes no allocator, a plugin whose process forbids
 * new device allocations, a fixed memory budget).  Runs one electromag2 shot,
 * in the two-pass form (cfg->flags must be 0 or SFD_FLAG_TWO_PASS), with the
 * whole device state in a file-scope device array of 32 MiB that every GPU
 * loading this library holds until exit; larger configurations are rejected
 * with SFD_ERR_BAD_ARG.  The array is taken from a device's memory when the
 * first call there loads its module (lazy module loading; at library load
 * with CUDA_MODULE_LOADING=EAGER), so that first call can fail with
 * SFD_ERR_CUDA on a full device: make it early, before the caller's own
 * memory budget is spent.  Inputs and outputs are host arrays: model
 * (6 planes as sfd_set_model), profiles (as sfd_set_cpml), source cell and
 * time functions (2 x nstep, as sfd_set_source), receivers (nrec (i,j,k)
 * triples) and traces out (nstep x 2 x nrec FP32).  Each call clears the
 * array first; calls whose GPU work overlaps race on it.  The first call on a
 * device looks up the array's address and should come before any stream
 * capture.  No counterpart in the reference: it is an addition for callers
 * that cannot allocate. */
int32_t sfd_electromag2_run_static(const sfd_config* cfg, const double* model, const double* profiles,
                                   int32_t isrc, int32_t ksrc, const double* srcfn, const int32_t* rec_ijk,
                                   float* traces, void* stream);

/* ---- Checkpoints ------------------------------------------------------------
 * The dynamic state (every field and CPML memory variable) of a handle,
 * copied to / from a caller-owned device buffer on the handle's stream.
 * Loading also sets the step counter (the source index). */
int32_t sfd_checkpoint_bytes(const sfd_handle* h, size_t* bytes);
int32_t sfd_checkpoint_save(sfd_handle* h, void* dev_dst);
int32_t sfd_checkpoint_load(sfd_handle* h, const void* dev_src, int64_t step);
/* sfd_run(h, nsteps) that also saves a checkpoint before every `every`
 * steps: checkpoint q, the state at step (current + q * every), goes to
 * dev_ckpt + q * stride (stride >= sfd_checkpoint_bytes, 4-byte aligned),
 * for q = 0 .. ceil(nsteps / every) - 1.  An electromag2 handle whose runs
 * are on chip writes them from the one launch of the run, without stopping
 * it; the other handles stop every `every` steps to copy the state. */
int32_t sfd_run_checkpointed(sfd_handle* h, int64_t nsteps, void* dev_ckpt, size_t stride, int32_t every);

/* ---- Discrete adjoint (electromag2 single-pass handles; seismic2) ----------
 * Gradient of J with respect to the model planes, given dJ/d(trace)
 * (device FP32 [nstep][2][nrec]; for J = 1/2 sum (d - d_obs)^2 this is the
 * residual).  Usage: after a forward run that saved checkpoints every S
 * steps, call sfd_adjoint_begin once, then for each checkpoint from the last
 * to the first: sfd_checkpoint_load(h, ckpt, step), sfd_adjoint_segment(h,
 * steps of that segment).  Each segment recomputes its forward states from
 * the checkpoint and runs the adjoint steps backwards over them; on an
 * electromag2 handle whose runs are on chip (sfd_on_chip) both are one
 * launch per segment.  The workspace (sfd_adjoint_bytes) holds S+1 forward
 * states.  On chip, a neighbouring tile that does not answer within the
 * wait limit makes sfd_adjoint_gradient return SFD_ERR_TIMEOUT.
 * seismic2: any step form; the corrected physics with 1-D CPML profiles
 * (SFD_FLAG_LEGACY_QUIRKS and SFD_FLAG_CPML_2D are refused), any density
 * method, attenuation and stress sources.  Set the force source after the
 * model (its amplitude is divided by rho there) for the rho gradient to
 * include the source term.  No counterpart in the reference (SeidarT has no
 * adjoint). */
int32_t sfd_adjoint_bytes(const sfd_handle* h, int32_t seg_steps, size_t* bytes);
int32_t sfd_adjoint_begin(sfd_handle* h, void* dev_work, size_t bytes, int32_t seg_steps, const float* dev_resid);
int32_t sfd_adjoint_segment(sfd_handle* h, int64_t nsteps);
/* The recompute-free form (electromag2 and seismic2 handles whose runs are
 * on chip): after sfd_adjoint_begin with seg_steps >= n,
 * sfd_adjoint_record(h, n) is the forward run of n steps (receivers
 * recorded, the handle advanced as by sfd_run) that also keeps every step's
 * state in the workspace; fill the residual, then sfd_adjoint_segment(h, n)
 * right after it runs the adjoint sweep over those states without
 * recomputing them.  The workspace then holds n+1 states (about 6.7 MB each
 * on a 1040 x 540 electromag2 grid, 2.5 MB on a 440 x 240 seismic2 one).
 * On chip, a seismic2 segment's recompute is itself one launch. */
int32_t sfd_adjoint_record(sfd_handle* h, int64_t nsteps);
/* Host FP64 planes: electromag2 dJ/d(eps11 eps13 eps33 sig11 sig13 sig33),
 * 6*NX*NZ values; seismic2 dJ/d(c11 c13 c15 c33 c35 c55 rho gamma_x
 * gamma_z), 9*NX*NZ values. */
int32_t sfd_adjoint_gradient(sfd_handle* h, double* planes, int64_t count);

/* ---- Batched runs ----------------------------------------------------------
 * Many 2-D models (electromag2 shots, seismic2 models of any sizes, mixed)
 * advance together in one persistent cooperative kernel launch with a grid
 * barrier per time step.  Replaces the per-shot process loop of the driver
 * (src/seidart/simulations/common_offset.py:143-284, one seidartfdtd call per
 * source).  The handles must be single-pass 2-D handles on one stream with
 * model and CPML set; each keeps its own state, source, receivers and traces.
 * The batch needs a small device scratch buffer of sfd_batch_scratch_bytes. */
typedef struct sfd_batch_s sfd_batch;
int32_t sfd_batch_scratch_bytes(int32_t nmodels, size_t* bytes);
int32_t sfd_batch_create(sfd_handle* const* handles, int32_t nmodels, void* dev_scratch, size_t bytes,
                         sfd_batch** out);
/* Tile rows per thread (1, 2, 4) and resident blocks per SM of the launch. */
int32_t sfd_batch_set_tiling(sfd_batch* b, int32_t zb, int32_t blocks_per_sm);
/* Advance every model nsteps steps (asynchronous). */
int32_t sfd_batch_run(sfd_batch* b, int64_t nsteps);
/* Longest wait, in ns, of a block at the batch kernel's grid barrier; 0
 * restores the default, 2 s.  A wait that runs out makes every block leave
 * the kernel and sfd_batch_status return SFD_ERR_TIMEOUT. */
int32_t sfd_batch_set_wait_limit(sfd_batch* b, int64_t ns);
/* Test aid: with `on` != 0 the grid barrier waits for one block more than the
 * launch has, so every block's wait runs out after the limit and the run ends
 * with SFD_ERR_TIMEOUT.  0 restores normal runs. */
int32_t sfd_batch_test_stall_waits(sfd_batch* b, int32_t on);
/* Synchronise; SFD_ERR_TIMEOUT if the grid barrier gave up, SFD_ERR_UNSTABLE
 * (with *failed_model) if a model blew up. */
int32_t sfd_batch_status(sfd_batch* b, int32_t* failed_model);
int32_t sfd_batch_destroy(sfd_batch* b);

#ifdef __cplusplus
}
#endif

#endif /* SEIDART_GB300_H */
