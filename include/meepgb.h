/*
 * meepgb.h — C ABI of the GB300 FDTD stepping library (libmeepgb.so).
 *
 * The library steps one lifted MEEP simulation (real float32 fields, 3-D, UPML,
 * isotropic chi1inv, Lorentz/Drude poles, electric point/extended sources, DFT and
 * flux monitors) on one GPU. It owns no field memory: every array is allocated by the
 * caller (the Python host uses torch tensors) and passed in by device pointer. It
 * allocates nothing on the device at any point, so a caller may capture mgb_step in a
 * CUDA graph.
 *
 * Reference interface this replaces (file:line inside the reference project):
 *   - plan_fast_path(fields, pml, grid, sources, chunk_layout)  meep_gpu/fastpath.py:6986
 *       -> mgb_create: one plan per configuration freeze, refusals named in the error text.
 *   - FastPathPlan.dispatch(slot, fields) for the slots step_B, fill_B, update_H, step_D,
 *     fill_D, update_E, update_P (meep_gpu/fastpath.py:4631, slots :575) together with the
 *     driver's in-between passes zero_metal_B/D and the electric source deposit
 *     (meep_gpu/driver.py:3533-3585, sources.py:2400)
 *       -> mgb_step: the whole FdtdDriver.step() body for nsteps steps in two fused
 *          kernels per step (H-half, E-half), plus the monitor accumulation of
 *          FluxMonitor.update / DFTMonitor.update (meep_gpu/dft.py:3031, :2197) on
 *          decimated steps.
 *   - FluxMonitor.get_flux_spectrum / _integrate_flux  meep_gpu/dft.py:3090, :3107
 *       -> mgb_flux_spectrum.
 *   - invalidate_fast_path()  meep_gpu/driver.py:3321  -> mgb_destroy + mgb_create.
 *
 * Conventions: arrays are C-contiguous (nx, ny, nz), z fastest. Every entry point
 * returns MGB_OK (0) or a negative error code; mgb_last_error() describes the last
 * failure of the calling thread. No C++ exception crosses this boundary, and no entry
 * point synchronises the device.
 */
#ifndef MEEPGB_H
#define MEEPGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MGB_ABI_VERSION 4
#define MGB_MAX_POLES 8
#define MGB_MAX_MONITORS 16
#define MGB_MAX_MONITOR_COMPONENTS 6

enum {
  MGB_OK = 0,
  MGB_ERR_ARGUMENT = -1,    /* a null or inconsistent argument */
  MGB_ERR_CUDA = -2,        /* a CUDA runtime error (launch, configuration) */
  MGB_ERR_UNSUPPORTED = -3, /* a configuration this engine refuses by name */
  MGB_ERR_RANGE = -4        /* a step outside the uploaded source-word table */
};

/* One PML auxiliary array: a full (nx, ny, nz) volume of which only the cells whose
 * coordinate along `axis` lies in the membership runs [a0, a1) U [b0, b1) are ever read
 * or written (the rest is never touched, so it moves no bytes); full-volume storage
 * keeps its index the cell's own linear index. */
typedef struct mgb_aux {
  float* data; /* device; NULL when the run has no PML */
  int32_t axis;
  int32_t a0, a1, b0, b1;
} mgb_aux;

/* One Lorentz/Drude pole (MEEP's realnum constants). Polarization storage covers the
 * box desc.pbox only; sigma[c] == NULL means the pole does not drive component c. */
typedef struct mgb_pole {
  float two_minus_od, gamma1, omega0dtsqr, gamma1inv;
  const float* sigma[3]; /* device, box-shaped */
  float* p[3][2];        /* device, box-shaped, two rotating buffers */
} mgb_pole;

/* One DFT accumulator: cell-centred samples of `ncomp` components over a region.
 * comp[i]: 0..2 = Ex..Ez, 3..5 = Hx..Hz. acc layout: [ncomp][nfreq][2 (re, im)][cells],
 * cells in C order over the region. */
typedef struct mgb_monitor {
  int32_t region[6]; /* x0, x1, y0, y1, z0, z1 (half-open) */
  int32_t ncomp;
  int32_t comp[MGB_MAX_MONITOR_COMPONENTS];
  int32_t nfreq;
  int32_t decimation;
  double scale;         /* dt * decimation / sqrt(2 pi) */
  double dt;            /* time step (E sampled at step*dt, H at step*dt - dt/2) */
  const double* omega;  /* device [nfreq], 2 pi f */
  float* acc;           /* device */
} mgb_monitor;

/* MEEP's D and B conductivity (mp.Medium D_conductivity / B_conductivity and the graded
 * mp.Absorber), which replaces the curl update f -= curl of a lossy component by
 * f = ((condfac f) - curl) condinv (step_generic.cpp step_curl). Index [side][q]: side 0
 * is B (stepped in the H half), side 1 is D (the E half). Replaces the conductivity
 * volumes Fields.set_d_conductivity / set_b_conductivity install
 * (meep_gpu/fields.py:775, :822) and the conductive curl forms of
 * meep_gpu/stepping.py:2828 (_apply_conductive_update) and :2844
 * (_apply_conductive_pml_update). */
typedef struct mgb_conductivity {
  const float* condfac[2][3]; /* device volumes, 1 - sigma dt/2 in float32; NULL: lossless */
  const float* condinv[2][3]; /* device volumes, 1 / (1 + sigma dt/2) rounded once from double */
  /* With a PML (pml_active), per lossy component: */
  float* fcond[2][3]; /* the conductive-stage history, a full volume read and written on
                       * the dsig membership of the chunks that keep the conductivity */
  /* [lattice: 0 integer, 1 half-integer][axis]: the one-rank chunk of every stored row
   * (0 the low PML chunk, 1 the interior, 2 the high one), device, length of the axis */
  const int8_t* chunk_of[2][3];
  /* per lossy component, bit (x * 9 + y * 3 + z) set when the chunk with those pieces
   * keeps a conductivity array for it (some sample of its loop volume is nonzero) */
  uint32_t keeps[2][3];
} mgb_conductivity;

/* The ghost words of mirror-folded axes, built by the caller (see mgb_sim_desc.mirror).
 * [0]: the B ghosts (H half), [1]: the D ghosts (E half). Entry t of a list: the ghost's
 * cell offset, the offset of the stored word it images, and a code (bits 0-1 the
 * component 0..2, bit 2 negate, bit 3 zero: the ghost sits on a metallic wall of
 * another axis). Entries are independent (any order steps the same words); lists in
 * x-plane order of the ghost offsets let the x-range split fold each range's ghosts
 * with the range (mgb_set_split). saved[h]: device scratch of MGB_FOLD_WORDS * count[h]
 * floats, zeroed by the caller, where the library keeps each ghost's state from before
 * its half. */
#define MGB_FOLD_WORDS (2 + MGB_MAX_POLES)
typedef struct mgb_fold {
  int32_t count[2];
  const int32_t* ghost[2];
  const int32_t* image[2];
  const uint8_t* code[2];
  float* saved[2];
} mgb_fold;

typedef struct mgb_sim_desc {
  int32_t abi_version; /* MGB_ABI_VERSION */
  int32_t nx, ny, nz;  /* at least 1 each (an axis of one cell is periodic: MEEP's unit
                        * direction, the invariant z of a 2-D run), fewer than 2^31 cells */
  int32_t metallic[3]; /* 1: PEC walls on that axis; 0: periodic wrap */
  float dtdx;          /* float32(dt / dx) */
  int32_t pml_active;
  /* UPML coefficient vectors [lattice: 0 integer, 1 half-integer][axis], device,
   * length of the axis. Ignored when pml_active == 0. */
  const float* kms[2][3];
  const float* sinv[2][3];
  const float* kps[2][3];
  /* primary fields, full volumes. H holds every cell: outside each component's
   * own-axis integer PML membership MEEP's H is B's word (mu = 1), so B needs no
   * storage of its own there. */
  float* E[3];
  float* D[3];
  float* H[3];
  const float* inv_eps[3]; /* may alias one another */
  /* PML auxiliaries: B and f_w of H on each H component's own-axis integer membership,
   * f_w of E on the own-axis half membership, and the curl split-field fu of B (half
   * lattice) and D (integer lattice) on the dsigu membership. */
  mgb_aux B[3];
  mgb_aux fwH[3];
  mgb_aux fwE[3];
  mgb_aux fuB[3];
  mgb_aux fuD[3];
  /* polarization */
  int32_t npoles;
  int32_t pbox[6];
  mgb_pole poles[MGB_MAX_POLES];
  /* sources: nsrc points in deposit order, the electric ones (components 0..2, into D
   * in the E half) first and then the last nsrc_magnetic magnetic ones (components
   * 3..5, into B in the H half, MEEP's step_source(B) after step_B) */
  int32_t nsrc;
  const int64_t* src_cell; /* device, linear index into the component volume */
  const int32_t* src_comp; /* device, 0..2 (Dx..Dz) or 3..5 (Bx..Bz) */
  int32_t src_box[6];      /* bounding box of the electric points, half-open */
  /* monitors */
  int32_t nmonitors;
  mgb_monitor monitors[MGB_MAX_MONITORS];
  /* status word: the E half ORs 1 into it when it writes a NaN/Inf E; a tile kernel ORs
   * 2 when a wait for its own shared-memory copies exceeds its time limit (the kernel
   * then stops stepping instead of spinning); a contraction ORs 4 when its tensor-core
   * wait runs out; the wavefront kernel ORs 8 when a wait for the chunks it reads runs
   * out (every later item of that launch is skipped). */
  int32_t* status; /* device, may be NULL */
  /* D and B conductivity, NULL for a lossless run; the library keeps a copy. A run with
   * a conductivity steps with the generic kernels (family 0 or 4) and is refused by the
   * batch and the adjoint entry points. */
  const mgb_conductivity* conductivity;
  /* magnetic source points: the last nsrc_magnetic of the nsrc, and their bounding box
   * (half-open). */
  int32_t nsrc_magnetic;
  int32_t src_box_magnetic[6];
  /* Bloch-periodic complex runs (k_point != 0): a complex run is two plans, one over the
   * real parts (part 0) and one over the imaginary parts (part 1), stepped together by
   * mgb_step_pair. bloch_axes bit a: axis a (periodic) carries the phase
   * eikna[a] = bloch_phase[a][0] + i bloch_phase[a][1] (f(x + L) = eikna f(x)); the
   * partner arrays are the other part's E and H. Zero bloch_axes: no phase. */
  int32_t bloch_axes;
  int32_t part;
  double bloch_phase[3][2];
  const float* partner_E[3];
  const float* partner_H[3];
  /* mirror symmetry (MEEP's mp.Mirror): mirror[a] = +1 (even) or -1 (odd) folds axis a
   * about the plane at its stored cell 1 (MEEP's halve(): full - full/2 + 1 cells from
   * one cell below the plane); 0: no plane. full[a]: the unfolded cell count.
   * metallic[a] is the far face: 1 a metallic wall; 0 periodic, when the axis stores
   * one cell more (MEEP's big_corner plane, then the far ghost slot past the second
   * mirror at doubled full[a]). Cell 0 of every component with Yee shift 0 on a folded
   * axis is the plane's ghost, and on a periodic one the last slot of every component
   * with shift 1 the second mirror's: after each half's sources the library writes them
   * from their images with the component's parity (the `fold` lists) and steps their E
   * (H) from those words. Monitors read a ladder site the fold does not store from its
   * image. Folded runs are refused by the batch and the adjoint. */
  int32_t mirror[3];
  int32_t full[3];
  mgb_fold fold;
  /* bit a: axis a is translationally invariant (z of a 2-D run, x and y of a 1-D one;
   * one periodic cell each). A curl partner whose derivative lies along such an axis is
   * absent, as MEEP's step plan drops it (fields.cpp figure_out_step_plan): the curl is
   * dtdx * (g1s - g1) or (-dtdx) * (g2s - g2) instead of the full bracket. Such runs
   * take a generic kernel family (their own kernels, with the chosen launch shape) and are
   * refused by the tile kernels, the wavefront path, the batch and the adjoint. */
  int32_t invariant;
} mgb_sim_desc;

typedef struct mgb_sim mgb_sim;

/* Step the two parts of a Bloch-periodic complex run together, steps [first_step,
 * first_step + nsteps): per step the H half of `real` then of `imag`, the E half of each,
 * then each one's monitors (a half of one part reads the other part's fields across the
 * phased faces). Both plans need their source words installed. */
int mgb_step_pair(mgb_sim* real, mgb_sim* imag, int64_t first_step, int32_t nsteps, void* stream);

/* Version of this ABI (MGB_ABI_VERSION). */
int mgb_abi_version(void);

/* Test hook: the limit, in nanoseconds, of the FIRST bounded wait of later launches of the
 * TMA tile kernels (which = 0: their first shared-memory stage; family 1) or of the
 * tensor-core contraction (which = 1: its first phase tile's MMAs); 0 makes that wait give
 * up at once, a negative value restores the normal limit (the default). A wait that runs
 * out sets its status bit (2 for the tile kernels in the plan's status word, 4 for the
 * contraction) and the kernel leaves; every later wait, including the one that lets the
 * kernel's own copies or MMAs finish before it exits or frees tensor memory, keeps its
 * normal bound. Process-wide. No reference counterpart. */
int mgb_set_test_wait_limit(int32_t which, int64_t nanoseconds);

/* Validate a descriptor and make a plan from a copy of it. Replaces plan_fast_path
 * (meep_gpu/fastpath.py:6986); refusals return MGB_ERR_UNSUPPORTED with the reason. */
int mgb_create(const mgb_sim_desc* desc, mgb_sim** out);

/* Largest grid the kernels index (32-bit cell offsets): nx * ny * nz < 2^31. */
#define MGB_MAX_CELLS 2147483647LL

/* Launch shape of the step kernels: a (block_z x block_y) tile of (z, y) columns per CTA
 * marching over x_chunk planes of x. No reference counterpart: the reference launches a
 * fixed 1-D grid of 256 threads, one cell each (cuda_kernels/step_curl_kernels.py:788). */
int mgb_set_launch_shape(mgb_sim* sim, int block_z, int block_y, int x_chunk);

/* Install the float64 source-deposit words for steps [first_step, first_step+steps):
 * words is a device array [steps][nsrc]; borrowed until replaced. Row n holds each
 * electric point's A = real(amp * J(n dt + dt/2)) * dt and each magnetic point's
 * real(amp * J(n dt)) * dt (times its lossy component's condinv). */
int mgb_set_source_words(mgb_sim* sim, const double* words, int64_t first_step, int64_t steps);

/* Advance steps first_step .. first_step+nsteps-1 on `stream` (a cudaStream_t; NULL is
 * the legacy default stream). Replaces the body of FdtdDriver.step() (meep_gpu/driver.py
 * :3419-3596) and its dispatch consults. Asynchronous. */
int mgb_step(mgb_sim* sim, int64_t first_step, int32_t nsteps, void* stream);

/* Launch one part of step `step` on `stream`: part 0 the H half, 1 the E half, 2 the
 * monitor accumulation of every monitor due after that step (nothing if none is due).
 * mgb_step(sim, n, 1, s) is mgb_launch(sim, n, 0..2, s) in order. Used to time each
 * kernel on its own stream with events, and to capture steps into a CUDA graph. */
int mgb_launch(mgb_sim* sim, int64_t step, int32_t part, void* stream);

/* Reduce one flux monitor (its comp[] = Ea, Eb, Ha, Hb, the tangential pair of the
 * normal) to out[f] = sum_cells w * Re(Ea conj(Hb) - Eb conj(Ha)), float64, on the
 * device. weights: device float32 [cells]. Replaces FluxMonitor._integrate_flux
 * (meep_gpu/dft.py:3107) without the dA * weight scale, which the host applies. */
int mgb_flux_spectrum(mgb_sim* sim, int32_t monitor, const float* weights, double* out,
                      void* stream);

/* Add the field energy sum |E|^2 eps + |B|^2 over the grid (eps = 1 / inv_eps of each E
 * component; B the stored B word on each H component's own-axis membership, H's word
 * elsewhere) to *out (device double), in float64, on `stream`. Replaces
 * FdtdDriver._field_energy (meep_gpu/driver.py:3634), the scalar of the divergence guard
 * _DivergenceGuard (driver.py:747-792). Asynchronous. */
int mgb_field_energy(mgb_sim* sim, double* out, void* stream);

/* 1 when the plan steps with the TMA tile kernels, 0 when with the generic kernels (a z
 * extent that is not a multiple of 4, or MEEPGB_TILES=0 in the environment). */
int mgb_uses_tiles(mgb_sim* sim);

/* Choose the kernel family of both halves: 0 the generic kernels (plain loads), 1 the
 * tile kernels (TMA-staged shared-memory planes; needs a z extent that is a multiple of
 * 4), 2 the generic kernels with the next plane's loads issued ahead, 4 and 5 families 0
 * and 2 with each thread's x chunk prefetched into L2 before it marches (3, the
 * warp-specialized tile kernel, steps the E half only: see mgb_select_half). All
 * compute the same words; the autotuner picks the faster for a grid. A run with a
 * conductivity takes families 0 and 4 only. No reference counterpart (the reference's
 * dispatch arbiter picks among its own kernel tables, meep_gpu/dispatch_preference.py). */
int mgb_select_kernels(mgb_sim* sim, int32_t family);

/* Choose the family and launch shape of one half alone (part 0 the H half, 1 the E
 * half): family 0 generic, 1 tiles, 2 generic with the next plane's loads issued ahead,
 * 3 warp-specialized tiles (E half), 4 / 5 families 0 / 2 with the x chunk prefetched
 * into L2;
 * block_z x block_y cells per CTA (a multiple of 32, at most 256; the tile kernels'
 * block is fixed) and x_chunk planes per CTA. The halves are separate launches, so any
 * pair computes the same words. No reference counterpart. */
int mgb_select_half(mgb_sim* sim, int32_t part, int32_t family, int32_t block_z, int32_t block_y,
                    int32_t x_chunk);

/* ---- X-range split stepping ----------------------------------------------------------
 * Each half launched as `ranges` launches over consecutive ranges of x planes, on streams
 * of the plan (created here, released by mgb_destroy) ordered by events: the H half of a
 * range after the E half of the step before on it and the range above, the E half of a
 * range after the H half on it and the range below. The GPU then fills one launch's tail
 * with the next ready range and begins a step on the low ranges while the previous one
 * finishes the high ones. mgb_step forks the streams from its stream and joins them back
 * (monitor kernels run on it, joined before and forked after). Generic kernel families
 * only (the tile kernels step every plane in one launch); refused for Bloch phases or a
 * periodic x axis. On a folded run each range's half is followed on its stream by the
 * fold of the range's ghosts, which needs ghost lists in x-plane order with every image
 * in its ghost's plane (plane 2 for plane 0's ghosts of a folded x axis; mgb_create
 * records whether they are, mgb_set_split refuses them otherwise); with a folded x axis
 * and ranges under 3 planes mgb_step steps unsplit. No reference counterpart. */
#define MGB_MAX_SPLIT 16

/* Split each half into `ranges` (2..MGB_MAX_SPLIT) x-range launches; 0 or 1 switches the
 * split off. */
int mgb_set_split(mgb_sim* sim, int32_t ranges);

/* ---- Wavefront stepping --------------------------------------------------------------
 * Runs of steps in one persistent launch: resident CTAs take (step, half, x chunk, (y, z)
 * tile) items in a skewed order that lets `window` consecutive steps pass over a chunk
 * while its neighbourhood is in L2, each item starting when the chunks it reads are done
 * (per-chunk completion counters; every wait is bounded, status bit 8 when one runs out).
 * The words are those of the launch-per-half kernels. Runs end after each step on which a
 * monitor is due (the monitor kernels run between launches). For runs without mirror
 * folds, Bloch phases or a conductivity, on a metallic x axis. No reference counterpart:
 * the reference launches one kernel per slot and step. */

/* Bytes of the caller's wave buffer for chunks of x_chunk planes, blocks of `window`
 * steps (1..16) and runs of at most max_steps steps (0 for bad arguments). */
size_t mgb_wave_bytes(mgb_sim* sim, int32_t x_chunk, int32_t window, int32_t max_steps);

/* Step with the wavefront path from now on: the column marches of family 0 (plain loads) or
 * 2 (the next plane's loads issued ahead), block_z (a multiple of 32) x block_y columns per
 * tile, x_chunk planes per chunk; buffer (device, 256-byte aligned, at least
 * mgb_wave_bytes() bytes, owned by the caller and used by every later mgb_step). Its item
 * table is written on `stream`. buffer NULL switches the path off. */
int mgb_set_wave(mgb_sim* sim, int32_t family, int32_t block_z, int32_t block_y, int32_t x_chunk,
                 int32_t window, int32_t max_steps, void* buffer, size_t bytes, void* stream);

/* Release the plan (never the caller's arrays). */
void mgb_destroy(mgb_sim* sim);

/* Copy the last error message of the calling thread into buf (NUL-terminated). */
int mgb_last_error(char* buf, size_t size);

/* ---- Tensor-core DFT accumulation ---------------------------------------------------
 * A monitor in buffered mode stores the cell-centred samples of up to MGB_DFT_DEPTH
 * decimated steps and adds them to its accumulators in one contraction on the tcgen05
 * tensor cores (TF32 with the 3xTF32 split, float32 accuracy; phases formed in float64
 * as the step-by-step path forms them). Replaces DFTMonitor.update / FluxMonitor.update
 * (meep_gpu/dft.py:2197, :3031) for K steps at once; the words differ from the
 * step-by-step sums only by float32 rounding order. */
#define MGB_DFT_DEPTH 32
#define MGB_DFT_MAX_FREQ 512

/* Bytes of the phase-table scratch a contraction of nfreq frequencies needs (0 when nfreq
 * is outside 1..MGB_DFT_MAX_FREQ). */
size_t mgb_dft_scratch_bytes(int32_t nfreq);

/* Switch monitor `monitor` to buffered mode: samples is a device float32 buffer of
 * MGB_DFT_DEPTH x (ncomp * cells) words, scratch at least mgb_dft_scratch_bytes(nfreq)
 * bytes (both 16-byte aligned, owned by the caller, one scratch may serve every monitor
 * of the plan). samples == NULL switches back to step-by-step accumulation. Refused
 * while the monitor holds buffered samples. */
int mgb_set_dft_buffer(mgb_sim* sim, int32_t monitor, float* samples, void* scratch,
                       size_t scratch_bytes);

/* Add every buffered sample to its monitor's accumulators (mgb_flux_spectrum does this
 * for its monitor). Call before reading accumulators. Asynchronous on `stream`. */
int mgb_dft_flush(mgb_sim* sim, void* stream);

/* Component `comp` (its index in the monitor's comp list) of monitor `monitor` as
 * interleaved complex64 words (re, im) [nfreq][cells] into `dst` (device, 2 * nfreq *
 * cells floats), buffered samples added first; for a complex run, `imag` is the
 * imaginary-part plan and the words are acc_re + i acc_im as complex64 sums round them,
 * (re.re - im.im, re.im + im.re). imag NULL: a real run. Asynchronous on `stream`. */
int mgb_read_accumulator(mgb_sim* real, mgb_sim* imag, int32_t monitor, int32_t comp, float* dst,
                         void* stream);

/* Samples a monitor holds buffered (-1 for a bad argument). */
int32_t mgb_dft_pending(mgb_sim* sim, int32_t monitor);

/* One contraction: acc[2f + 0][n] += sum_k cos(w_f t_k) * scale * samples[k * ld + n],
 * acc[2f + 1][n] += the same with sin, for n < ncols, k < nsamples <= MGB_DFT_DEPTH,
 * t_k = (first_step + k * step_stride) * dt (less dt/2 when half_step_back), w = omega
 * (device float64 [nfreq]); acc is device float32 [2 nfreq][ncols]. scratch: device, at
 * least mgb_dft_scratch_bytes(nfreq) bytes, rewritten by every call. Asynchronous. */
int mgb_dft_contract(const float* samples, int64_t ld, int64_t ncols, int32_t nsamples,
                     const double* omega, int32_t nfreq, int64_t first_step, int32_t step_stride,
                     double dt, int32_t half_step_back, double scale, float* acc, void* scratch,
                     size_t scratch_bytes, void* stream);

/* mgb_dft_contract with no scratch argument and no allocation: the phase table lives in
 * a device array of the library sized for MGB_DFT_MAX_FREQ frequencies (looked up once
 * per device). Every refusal (sizes beyond the maximum, ld < ncols, a null argument), and
 * a call with no work (nsamples or ncols 0), returns before the device is touched. Calls
 * that overlap on the device share that table and race: order them on one stream. */
int mgb_dft_contract_noalloc(const float* samples, int64_t ld, int64_t ncols, int32_t nsamples,
                             const double* omega, int32_t nfreq, int64_t first_step,
                             int32_t step_stride, double dt, int32_t half_step_back, double scale,
                             float* acc, void* stream);

/* Status word of the standalone contractions (mgb_dft_contract, mgb_dft_contract_noalloc)
 * on the current device: a device int of the library, ORed with 4 when a contraction's
 * tensor-core wait ran out (that call left the accumulators as they were, or added only
 * the phase tiles before the one that timed out). It stays set until cleared. Queues a
 * copy of the word into dst (device memory, or page-locked host memory; 4 bytes) on
 * `stream` and, when clear is nonzero, a reset to zero after it. Asynchronous; allocates
 * nothing. No reference counterpart (the reference's kernels report no wait). */
int mgb_dft_contract_status(int32_t* dst, int32_t clear, void* stream);

/* ---- Adjoint (reverse-time) stepping ------------------------------------------------
 * No reference counterpart (the reference has no adjoint). The adjoint state is a second
 * plan made by mgb_create over adjoint arrays laid out as the forward's (E, D, H and the
 * PML auxiliaries), with the forward's coefficient tables, memberships and inverse
 * permittivity, no sources or poles, and the objective's monitor whose acc points at the
 * objective's derivative with respect to the monitor's accumulators. */
typedef struct mgb_adjoint {
  float* mu_b[3];       /* device volumes: adjoint of the H half's curl input */
  float* mu_d[3];       /* device volumes: adjoint of the E half's curl input */
  int32_t box[6];       /* gradient box (half-open cell ranges x, y, z) */
  const float* d_after; /* device [3][box cells]: forward D after the step being reversed */
  float* grad_inv;      /* device [box cells]: += dJ/d(inverse permittivity) */
} mgb_adjoint;

/* Reverse forward step `step`: the transposed E half (with the gather of mu_b left by
 * the reversal of step + 1, and the gradient over the box), then the transposed H half.
 * mu_b must be zero before the reversal of the last step. Asynchronous. */
int mgb_adjoint_step(mgb_sim* adj, const mgb_adjoint* a, int64_t step, void* stream);

/* Add the adjoint of the monitor's sample taken after step post - 1 (due when post is a
 * multiple of its decimation) into the adjoint E and H. Asynchronous. */
int mgb_adjoint_inject(mgb_sim* adj, int32_t monitor, int64_t post, void* stream);

/* One checkpoint interval in one call: the forward plan (restored to the state before
 * first_step by the caller) steps first_step .. first_step+nsteps-1 again (H and E halves,
 * no monitors), saving D over the box after each step into d_history [nsteps][3][box
 * cells]; then the adjoint steps back through the same steps, with the adjoint of every
 * sample of monitor `monitor` added where the forward took one. The forward plan's
 * source words must cover the interval. Asynchronous. */
int mgb_adjoint_segment(mgb_sim* fwd, mgb_sim* adj, const mgb_adjoint* a, int64_t first_step,
                        int32_t nsteps, int32_t monitor, float* d_history, void* stream);

/* Copy [3][box cells] of a plan's E (family 0), D (1) or H (2) into dst. Asynchronous. */
int mgb_copy_box(mgb_sim* sim, int32_t family, const int32_t* box, float* dst, void* stream);

/* ---- Batched stepping of independent simulations (serving) ---------------------------
 * No reference counterpart: the reference steps one simulation per process
 * (meep_gpu/driver.py:3419, one FdtdDriver per GPU, README.md:127). A batch is a slot
 * table over plans created with mgb_create; every step of mgb_batch_step advances each
 * active slot that has steps left by one, in kernels shared by all slots (one CTA per
 * work item), so simulations of different sizes step together. A slot's words equal
 * those of the same plan stepped alone. The caller owns every device array, the batch's
 * tables included. */
typedef struct mgb_batch mgb_batch;

/* Bytes of the device buffer that holds a batch's tables: max_slots slots, max_work step
 * items and max_dft_work monitor items (256 cells each). */
size_t mgb_batch_bytes(int32_t max_slots, int32_t max_work, int32_t max_dft_work);

/* Create a batch over a caller-allocated, 256-byte aligned device buffer of at least
 * mgb_batch_bytes() bytes. */
int mgb_batch_create(int32_t max_slots, int32_t max_work, int32_t max_dft_work,
                     void* device_buffer, size_t bytes, mgb_batch** out);

/* Set the batch's launch shape: block_z (a multiple of 32) x block_y cells per CTA,
 * block_z * block_y <= 256, x_chunk x cells per step item. Takes effect at the next
 * mgb_batch_commit. The default is 32 x 4 x 4. */
int mgb_batch_set_shape(mgb_batch* batch, int32_t block_z, int32_t block_y, int32_t x_chunk);

/* Set the marches the step items run: family 2 (the prefetching marches, the default)
 * or 4 (the generic marches with each item's x chunk prefetched into L2). Takes effect
 * at the next mgb_batch_step (a captured graph is rebuilt). */
int mgb_batch_set_family(mgb_batch* batch, int32_t family);

/* Put a plan in a slot, to run steps 0 .. end_step-1 from its arrays' current words
 * (normally zero). words: device float64 [end_step][points] deposit words of its sources
 * (electric and magnetic points, the plan's order) from step 0 (NULL if it has none); the
 * plan's own mgb_set_source_words table is not used. At most 2 monitors of at most 512
 * frequencies. The two parts of a Bloch-phased complex run go in two slots of the same
 * batch. Refused: a conductivity, mirror folds. Takes effect at the next
 * mgb_batch_commit; the plan and its arrays must outlive the slot's last queued step. */
int mgb_batch_set_slot(mgb_batch* batch, int32_t slot, mgb_sim* sim, int64_t end_step,
                       const double* words);

/* Empty a slot (takes effect at the next mgb_batch_commit). */
int mgb_batch_clear_slot(mgb_batch* batch, int32_t slot);

/* Upload the changed slots and the rebuilt work lists on `stream` (stream-ordered after
 * the batch steps queued before). */
int mgb_batch_commit(mgb_batch* batch, void* stream);

/* Queue nsteps batch steps on `stream`: plain launches (use_graph 0) or one replay of a
 * CUDA graph of nsteps steps (use_graph 1), captured on first use and again only when
 * nsteps, the stream or the launch shape change. Slots coming and going need no
 * recapture: the captured launches' grid sizes are updated in the executable graph.
 * Asynchronous; the slots' step counters advance on the host at once. */
int mgb_batch_step(mgb_batch* batch, int32_t nsteps, int32_t use_graph, void* stream);

/* Every slot's step once the queued batch steps have run (-1 for an empty slot) into
 * steps[max_slots]. A slot has run all its steps when this equals its end_step; its
 * results are in its arrays once the stream has passed the queued steps. No device
 * access. */
int mgb_batch_steps(mgb_batch* batch, int64_t* steps);

/* Committed step items (which = 0) or monitor items (which = 1). */
int64_t mgb_batch_items(mgb_batch* batch, int32_t which);

/* Release the batch (never the caller's buffer or plans). */
void mgb_batch_destroy(mgb_batch* batch);

#ifdef __cplusplus
}
#endif

#endif /* MEEPGB_H */
