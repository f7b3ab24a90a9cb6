// Device side of one FDTD step, shared by the launch-per-half kernels (meepgb.cu) and
// the persistent wavefront kernel (wave.cu): the step parameters, the per-cell updates of
// the H and E halves (MEEP's step_B / update_H / step_D / update_E / update_P forms, in the
// reference's float32 operation order) and the column marches over x that apply them.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "meepgb.h"

namespace mgbstep {

constexpr int kInteger = 0;
constexpr int kHalf = 1;

// ------------------------------------------------------------------------------------
struct StepParams {
  int nx, ny, nz;
  int pml;  // 1 when the run has an absorber (the PML memberships below are live)
  // The box outside every membership of every auxiliary (x0, x1, y0, y1, z0, z1): a CTA
  // whose cells all lie in it steps the plain update (no membership tests, no tables).
  int inner[6];
  int met[3];
  float dtdx;
  const float* kms[2][3];
  const float* sinv[2][3];
  const float* kps[2][3];
  float* E[3];
  float* D[3];
  float* H[3];
  const float* inv_eps[3];
  mgb_aux B[3], fwH[3], fwE[3], fuB[3], fuD[3];
  int npoles;
  int pbox[6];
  mgb_pole poles[MGB_MAX_POLES];
  int nsrc;                 // every point; the last nsrc_h are magnetic (into B)
  const int64_t* src_cell;
  const int32_t* src_comp;
  int src_box[6];           // box of the electric points
  const double* src_words;  // row for the current step, [nsrc]
  int nsrc_h;
  int src_box_h[6];         // box of the magnetic points
  int32_t* status;
  int l2pf;  // 1: each thread prefetches its x chunk's field planes into L2 before marching
  int xbase; // first x chunk of a launch that covers a range of the planes (0: from plane 0)
  // Bloch phases (complex runs with k != 0): per axis 0 none, 1 copy, 2 negate, 3 the
  // phase (re, im) rounded to float32; `part` 0 steps real parts, 1 imaginary parts;
  // pE / pH the other part's E and H
  int bloch;
  int bmode[3];
  float bre[3], bim[3];
  int part;
  const float* pE[3];
  const float* pH[3];
  // bit a: axis a is translationally invariant (a 2-D or 1-D run): curl partners whose
  // derivative lies along it are absent (curl_term)
  int inv;
};

// One curl bracket, dtdx * (((S1 - A1) + A2) - S2) (S the shifted operand, A the one at
// the cell, the partners in MEEP's order), with MEEP's step plan on a reduced-dimension
// run (fields.cpp figure_out_step_plan, step_generic.cpp step_curl): a partner whose
// derivative axis the run does not resolve is absent, and the one-partner forms are
// dtdx * (S1 - A1) and (-dtdx) * (S2 - A2) rather than the full bracket, which rounds
// differently where the absent partner is nonzero. axis1 / axis2: the partners'
// derivative axes.
// RED: the march of a reduced-dimension run (the kernels send such runs to one general
// march compiled with it); the 3-D marches compile the full bracket alone, since the
// branches below, inlined into every march, cost them registers (the H march spilled
// 128 bytes a thread instead of 4).
template <bool RED>
__device__ __forceinline__ float curl_term(const StepParams& p, float s1, float a1, float a2, float s2,
                                           int axis1, int axis2) {
  if (!RED || p.inv == 0) return p.dtdx * (((s1 - a1) + a2) - s2);
  const bool have1 = ((p.inv >> axis1) & 1) == 0, have2 = ((p.inv >> axis2) & 1) == 0;
  if (have1 && have2) return p.dtdx * (((s1 - a1) + a2) - s2);
  if (have1) return p.dtdx * (s1 - a1);
  if (have2) return (-p.dtdx) * (s2 - a2);
  return 0.f;
}

// The ghost lists of mirror-folded axes (mgb_fold), passed to the fold kernels.
struct FoldArgs {
  int count[2];
  const int32_t* ghost[2];
  const int32_t* image[2];
  const uint8_t* code[2];
  float* saved[2];
  // the entries [lo, hi) of each list a launch takes (the whole lists, or one x range's)
  int lo[2];
  int hi[2];
};

// Tensor maps of the tile kernels (each 64-byte aligned, passed as __grid_constant__).
struct TileMaps {
  CUtensorMap E[3];     // box 68 x 9 x 1 (halo above in z and y)
  CUtensorMap Hown[3];  // box 64 x 8 x 1
  CUtensorMap Hhalo[3]; // box 68 x 9 x 1 (halo below in z and y)
  CUtensorMap D[3];     // box 64 x 8 x 1
  CUtensorMap inv[3];   // box 64 x 8 x 1
  int ninv;             // distinct inverse-epsilon volumes (1 or 3)
  int inv_of[3];        // which of inv[] serves each component
  int stages;
  long long first_wait_ns;  // limit of the first stage wait; negative: the normal limit
                            // (a test hook: 0 gives up before waiting)
};

struct BoxArgs {
  int box[6];
  float* dst;
};

struct DftParams {
  int nx, ny, nz;
  int met[3];
  const float* E[3];
  const float* H[3];
  mgb_monitor mon;
  // Bloch phases as in StepParams (a sample at ladder index 0 of a phased axis is the
  // stored word times conj(eikna) there)
  int bloch;
  int bmode[3];
  float bre[3], bim[3];
  int part;
  const float* pE[3];
  const float* pH[3];
  // mirror folds: bit a of `fold` folds axis a (full[a] unfolded cells), of `far` when
  // its outer face is periodic (a second mirror at doubled full[a]); bit a of neg[comp]
  // says the component is odd about that plane
  int fold;
  int far;
  int full[3];
  int neg[6];
};

__device__ __forceinline__ bool in_runs(const mgb_aux& a, int x) {
  return (x >= a.a0 && x < a.a1) || (x >= a.b0 && x < a.b1);
}

__device__ __forceinline__ float ldgf(const float* base, int at) { return __ldg(base + at); }

// A curl operand read across a Bloch-phased face at the same stored index (MEEP's
// not-owned word): the stored word of this part (`own`) and of the other part
// (`partner[c]`) times the axis's phase, conjugated for the word below the window
// (`conj`), each product and sum rounded on its own: copy within 1e-13 of +1, negation
// within 1e-13 of -1, else re = (a*re) - (b*im), im = (a*im) + (b*re).
template <typename P>
__device__ __forceinline__ float bloch_word(const P& p, int axis, bool conj, float own, const float* partner,
                                            long long c) {
  const int mode = p.bmode[axis];
  if (mode == 2) return -own;
  if (mode != 3) return own;
  const float a = p.bre[axis];
  const float b = conj ? -p.bim[axis] : p.bim[axis];
  const float other = partner[c];
  return p.part ? (a * own) + (b * other) : (a * own) - (b * other);
}

// Entry of a step kernel launched as its stream predecessor's programmatic dependent:
// let this grid's own dependent be scheduled once every CTA here has started (its CTAs
// then take the SM slots this grid's last wave frees, and wait), then wait for the
// predecessor grid to complete with its memory visible, before any global access. In a
// launch without the programmatic attribute both instructions do nothing.
__device__ __forceinline__ void step_entry() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

__device__ __forceinline__ void l2_prefetch(const float* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Prefetch into L2 the words of `count` planes (stride sx) from offset c of the first
// `nvol` of NV volumes: the march's later loads then find them in L2. Lane-wise, so a
// warp's 32 z cells make one line per volume and plane.
template <int NV>
__device__ __forceinline__ void prefetch_planes(const float* const (&vols)[NV], int nvol, int c, int sx, int count) {
  for (int t = 0; t < count; ++t) {
#pragma unroll
    for (int v = 0; v < NV; ++v)
      if (v < nvol) l2_prefetch(vols[v] + c + t * sx);
  }
}

// ---- per-cell updates ----------------------------------------------------------------
//
// Component q's curl update uses the split-field recurrence where its dsigu membership
// holds (dsig = axis q+1, dsigu = axis q+2, MEEP's cycle X -> Y -> Z):
//   fu' = ((kms*fu) - curl)*sinv;  f' = (((kms_u*f) + fu') - fu)*sinv_u
// and f' = ((kms*f) - curl)*sinv elsewhere. The constitutive accumulation on the own-
// axis membership is f_w' = src, f' = f + ((kps*src) - (kms*f_w)).
//
// Every PML coefficient outside its membership is exactly 1 (checked when the tables are
// built), so a cell outside all six memberships steps f - curl and H = B: the same
// words. A warp takes that fast path when none of its lanes is in a membership (the
// lanes of a warp share y and the plane, so only the z lanes can differ).
//
// Coefficients and membership flags depend on one coordinate each. A thread keeps y and
// z fixed while it marches over x, so everything indexed by j or k is formed once per
// thread (a "column") and everything indexed by i once per plane.

// H half: B lives on the half lattice transversally (curl tables), H on the integer
// lattice of its own axis (constitutive tables).
struct HColumn {
  bool f0, f2, b1, b2;                  // fuB[0] (z), fuB[2] (y), B[1] (y), B[2] (z)
  float kms_yh, sinv_yh, kps_y, kms_y;  // j-indexed
  float kms_zh, sinv_zh, kps_z, kms_z;  // k-indexed
};
struct HPlane {
  bool f1, b0;                          // fuB[1] (x), B[0] (x)
  float kms_xh, sinv_xh, kps_x, kms_x;
};

__device__ __forceinline__ HColumn h_column(const StepParams& p, int j, int k) {
  HColumn c;
  c.f0 = in_runs(p.fuB[0], k); c.f2 = in_runs(p.fuB[2], j);
  c.b1 = in_runs(p.B[1], j); c.b2 = in_runs(p.B[2], k);
  c.kms_yh = ldgf(p.kms[kHalf][1], j); c.sinv_yh = ldgf(p.sinv[kHalf][1], j);
  c.kps_y = ldgf(p.kps[kInteger][1], j); c.kms_y = ldgf(p.kms[kInteger][1], j);
  c.kms_zh = ldgf(p.kms[kHalf][2], k); c.sinv_zh = ldgf(p.sinv[kHalf][2], k);
  c.kps_z = ldgf(p.kps[kInteger][2], k); c.kms_z = ldgf(p.kms[kInteger][2], k);
  return c;
}

__device__ __forceinline__ HPlane h_plane(const StepParams& p, int i) {
  HPlane c = {};
  c.f1 = in_runs(p.fuB[1], i); c.b0 = in_runs(p.B[0], i);
  return c;
}

// The plane's coefficients, needed only on the PML path.
__device__ __forceinline__ void h_plane_coefficients(const StepParams& p, int i, HPlane& c) {
  c.kms_xh = ldgf(p.kms[kHalf][0], i); c.sinv_xh = ldgf(p.sinv[kHalf][0], i);
  c.kps_x = ldgf(p.kps[kInteger][0], i); c.kms_x = ldgf(p.kms[kInteger][0], i);
}

// One curl component. DSIG: a lane of the warp may sit in the dsig membership (else the
// dsig coefficients are exactly 1 for the whole warp and drop out); DSIGU: a lane may sit
// in the dsigu membership (`member` says whether this one does), which selects the
// split-field recurrence and its auxiliary `u` (the new one returned in `n`).
template <bool DSIG, bool DSIGU>
__device__ __forceinline__ float curl_form(float f, float curl, bool member, float u, float kms,
                                           float sinv, float kms_u, float sinv_u, float& n) {
  if (DSIGU && member) {
    n = DSIG ? (kms * u - curl) * sinv : u - curl;
    return ((kms_u * f + n) - u) * sinv_u;
  }
  return DSIG ? (kms * f - curl) * sinv : f - curl;
}

// One curl component of a lossy side (MEEP's step_curl with a conductivity, restated
// from meep_gpu/stepping.py:2828 and :2844). `side` 0 is B, 1 is D; `sg` / `su` whether
// the cell's chunk carries the component's dsig / dsigu layer. With cf = condfac and
// ci = condinv, in float32 in this order:
//   no PML:                 f' = ((cf*f) - curl)*ci
//   a chunk that keeps the component's conductivity, dsig and dsigu:
//     g' = ((cf*g) - curl)*ci (the conductive-stage history g), u' = ((kms*u) + (g' - g))*sinv,
//     f' = (((kms_u*f) + u') - u)*sinv_u
//   dsig only: g' as above, f' = ((kms*f) + (g' - g))*sinv
//   dsigu only: u' = ((cf*u) - curl)*ci, f' = (((kms_u*f) + u') - u)*sinv_u
//   neither: f' = ((cf*f) - curl)*ci
//   a chunk that keeps none: the lossless forms of curl_form.
// A component without a conductivity takes curl_form. The increment (g' - g) is formed
// before it is added, as MEEP groups it.
template <bool PML>
__device__ __forceinline__ float cond_curl(const mgb_conductivity& cp, int side, int q, int i, int j, int k,
                                           int c, float f, float curl, bool sg, bool su, float u, float kms,
                                           float sinv, float kms_u, float sinv_u, float& n) {
  const float* fac = cp.condfac[side][q];
  if (fac == nullptr) return curl_form<PML, PML>(f, curl, su, u, kms, sinv, kms_u, sinv_u, n);
  const float cf = __ldg(fac + c);
  const float ci = __ldg(cp.condinv[side][q] + c);
  if (!PML) return ((cf * f) - curl) * ci;
  // the chunk of this cell: per axis, the piece on the component's lattice there (B sits
  // on the integer lattice of its own axis and the half lattice of the others, D the
  // other way round)
  const int own = side == 0 ? kInteger : kHalf, other = side == 0 ? kHalf : kInteger;
  const int px = __ldg(cp.chunk_of[q == 0 ? own : other][0] + i);
  const int py = __ldg(cp.chunk_of[q == 1 ? own : other][1] + j);
  const int pz = __ldg(cp.chunk_of[q == 2 ? own : other][2] + k);
  if (((cp.keeps[side][q] >> (px * 9 + py * 3 + pz)) & 1u) == 0)
    return curl_form<true, true>(f, curl, su, u, kms, sinv, kms_u, sinv_u, n);
  if (sg) {
    float* hist = cp.fcond[side][q] + c;
    const float g = *hist;
    const float g_new = ((cf * g) - curl) * ci;
    *hist = g_new;
    const float inc = g_new - g;
    if (su) {
      n = ((kms * u) + inc) * sinv;
      return (((kms_u * f) + n) - u) * sinv_u;
    }
    return ((kms * f) + inc) * sinv;
  }
  if (su) {
    n = ((cf * u) - curl) * ci;
    return (((kms_u * f) + n) - u) * sinv_u;
  }
  return ((cf * f) - curl) * ci;
}

// B from its curls, zero_metal_B, H from B (update_H) for one cell at offset c, and the
// auxiliary stores, for a warp that may touch the x (SX), y (SY) and z (SZ) memberships.
// Each axis switches on one feature per component (x: Bx own, By dsigu, Bz dsig;
// y: Bx dsig, By own, Bz dsigu; z: Bx dsigu, By dsig, Bz own). `h_old` is the stored H
// word (the old B outside the own-axis membership).
// Every auxiliary word an H cell reads, loaded from the membership flags alone, so the
// caller issues these loads together with the field loads (one round trip per plane).
struct HAux {
  float b[3], u[3];
};

__device__ __forceinline__ void h_aux_load(const StepParams& p, const HColumn& col, const HPlane& pl, int c,
                                           HAux& a) {
  const bool sb[3] = {pl.b0, col.b1, col.b2};
  const bool sf[3] = {col.f0, pl.f1, col.f2};
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    a.b[q] = sb[q] ? p.B[q].data[c] : 0.f;
    a.u[q] = sf[q] ? p.fuB[q].data[c] : 0.f;
  }
}

template <bool SX, bool SY, bool SZ, bool COND = false, bool MSRC = false>
__device__ __forceinline__ void h_cell_v(const StepParams& p, const HColumn& col,
                                         const HPlane& pl, int first_step, int c, float cx,
                                         float cy, float cz, const float h_old[3], const HAux& a,
                                         float h_new[3], const mgb_conductivity* cp = nullptr,
                                         int i = 0, int j = 0, int k = 0) {
  const bool sb0 = SX && pl.b0, sb1 = SY && col.b1, sb2 = SZ && col.b2;
  const bool sf0 = SZ && col.f0, sf1 = SX && pl.f1, sf2 = SY && col.f2;
  // The cell's auxiliary words (loaded by the caller, before any store).
  float b0 = sb0 ? a.b[0] : h_old[0];
  float b1 = sb1 ? a.b[1] : h_old[1];
  float b2 = sb2 ? a.b[2] : h_old[2];
  // f_w of H: MEEP's update_H stores B's new word in it on the own-axis membership, where
  // B itself is stored too, so after step 0 (which reads neither) it is always B's old
  // word: read once, as B, and not stored separately
  const float w0 = a.b[0], w1 = a.b[1], w2 = a.b[2];
  const float u0 = a.u[0], u1 = a.u[1], u2 = a.u[2];
  // Bx: dsig y, dsigu z; By: dsig z, dsigu x; Bz: dsig x, dsigu y.
  float n0 = 0.f, n1 = 0.f, n2 = 0.f;
  if (COND) {
    // the dsig membership of each component is the dsigu membership of the component
    // two after it (same axis, same lattice)
    constexpr bool P = SX || SY || SZ;
    b0 = cond_curl<P>(*cp, 0, 0, i, j, k, c, b0, cx, col.f2, sf0, u0, col.kms_yh, col.sinv_yh, col.kms_zh, col.sinv_zh, n0);
    b1 = cond_curl<P>(*cp, 0, 1, i, j, k, c, b1, cy, col.f0, sf1, u1, col.kms_zh, col.sinv_zh, pl.kms_xh, pl.sinv_xh, n1);
    b2 = cond_curl<P>(*cp, 0, 2, i, j, k, c, b2, cz, pl.f1, sf2, u2, pl.kms_xh, pl.sinv_xh, col.kms_yh, col.sinv_yh, n2);
  } else {
    b0 = curl_form<SY, SZ>(b0, cx, sf0, u0, col.kms_yh, col.sinv_yh, col.kms_zh, col.sinv_zh, n0);
    b1 = curl_form<SZ, SX>(b1, cy, sf1, u1, col.kms_zh, col.sinv_zh, pl.kms_xh, pl.sinv_xh, n1);
    b2 = curl_form<SX, SY>(b2, cz, sf2, u2, pl.kms_xh, pl.sinv_xh, col.kms_yh, col.sinv_yh, n2);
  }
  // Magnetic sources at t (MEEP's step_source(B) right after step_B): the same double
  // subtract into B, before zero_metal_B and update_H.
  if (MSRC && i >= p.src_box_h[0] && i < p.src_box_h[1] && j >= p.src_box_h[2] &&
      j < p.src_box_h[3] && k >= p.src_box_h[4] && k < p.src_box_h[5]) {
    for (int s = p.nsrc - p.nsrc_h; s < p.nsrc; ++s) {
      if (p.src_cell[s] != c) continue;
      const int q = p.src_comp[s];
      const double w = p.src_words[s];
      if (q == 3) b0 = __double2float_rn(__dsub_rn((double)b0, w));
      else if (q == 4) b1 = __double2float_rn(__dsub_rn((double)b1, w));
      else b2 = __double2float_rn(__dsub_rn((double)b2, w));
    }
  }
  // zero_metal_B happens in the caller before this returns its words (masks above).
  h_new[0] = b0; h_new[1] = b1; h_new[2] = b2;
  // update_H on the own-axis integer membership (MEEP starts H and f_w from B once).
  if (SX && sb0) h_new[0] = (first_step ? b0 : h_old[0]) + (pl.kps_x * b0 - pl.kms_x * (first_step ? b0 : w0));
  if (SY && sb1) h_new[1] = (first_step ? b1 : h_old[1]) + (col.kps_y * b1 - col.kms_y * (first_step ? b1 : w1));
  if (SZ && sb2) h_new[2] = (first_step ? b2 : h_old[2]) + (col.kps_z * b2 - col.kms_z * (first_step ? b2 : w2));
  if (sf0) p.fuB[0].data[c] = n0;
  if (sf1) p.fuB[1].data[c] = n1;
  if (sf2) p.fuB[2].data[c] = n2;
  if (sb0) p.B[0].data[c] = b0;
  if (sb1) p.B[1].data[c] = b1;
  if (sb2) p.B[2].data[c] = b2;
}

// Whether the H variant chosen for `axes` reads the plane's x coefficients (every
// variant but the plain one and the z-only one does).
__device__ __forceinline__ bool h_needs_plane(int axes) { return axes != 0 && axes != 4; }

// One cell of the H half: masks, the variant for the warp's memberships, zero_metal_B.
// `axes` bit 0/1/2: the warp touches the x/y/z memberships (0 on the fast path).
template <bool PML, bool COND = false, int AX = -1, bool MSRC = false>
__device__ __forceinline__ void h_cell(const StepParams& p, const HColumn& col, const HPlane& pl,
                                       int axes, int first_step, int i, int j, int k, int c,
                                       float cx, float cy, float cz, const float h_old[3],
                                       const HAux& a, float h_new[3], const mgb_conductivity* cp = nullptr) {
  if (p.met[0] && i == 0) cx = 0.f;
  if (p.met[1] && j == 0) cy = 0.f;
  if (p.met[2] && k == 0) cz = 0.f;
  // zero_metal_B clears the wall samples after the curl update; a wall cell is never
  // in its component's own-axis membership, so there H is B and clearing H_new after
  // the accumulation is the same word.
  if (COND) {
    // a lossy run: the variant of the CTA's axes, or the general one (the conductive
    // forms test each membership per cell)
    constexpr bool X = AX < 0 || (AX & 1), Y = AX < 0 || (AX & 2), Z = AX < 0 || (AX & 4);
    if (PML) h_cell_v<X, Y, Z, true, MSRC>(p, col, pl, first_step, c, cx, cy, cz, h_old, a, h_new, cp, i, j, k);
    else h_cell_v<false, false, false, true, MSRC>(p, col, pl, first_step, c, cx, cy, cz, h_old, a, h_new, cp, i, j, k);
  } else if (PML && AX >= 0) {
    // the CTA's memberships are known: exactly the variant of its axes
    h_cell_v<(AX & 1) != 0, (AX & 2) != 0, (AX & 4) != 0, false, MSRC>(p, col, pl, first_step, c, cx, cy, cz, h_old,
                                                                        a, h_new, nullptr, i, j, k);
  } else if (!PML || axes == 0) {
    h_cell_v<false, false, false, false, MSRC>(p, col, pl, first_step, c, cx, cy, cz, h_old, a, h_new, nullptr, i, j, k);
  } else {
    // The z-only edge (the two z-edge warps of every interior row) is the commonest slow
    // case; every other mix takes the general variant.
    if (axes == 4)
      h_cell_v<false, false, true, false, MSRC>(p, col, pl, first_step, c, cx, cy, cz, h_old, a, h_new, nullptr, i, j, k);
    else
      h_cell_v<true, true, true, false, MSRC>(p, col, pl, first_step, c, cx, cy, cz, h_old, a, h_new, nullptr, i, j, k);
  }
  if (p.met[0] && i == 0) h_new[0] = 0.f;
  if (p.met[1] && j == 0) h_new[1] = 0.f;
  if (p.met[2] && k == 0) h_new[2] = 0.f;
}

// E half: D lives on the integer lattice transversally (curl tables), E on the half
// lattice of its own axis (constitutive tables).
struct EColumn {
  bool f0, f2, w1, w2;                  // fuD[0] (z), fuD[2] (y), fwE[1] (y), fwE[2] (z)
  float kms_y, sinv_y, kps_yh, kms_yh;  // j-indexed
  float kms_z, sinv_z, kps_zh, kms_zh;  // k-indexed
};
struct EPlane {
  bool f1, w0;                          // fuD[1] (x), fwE[0] (x)
  float kms_x, sinv_x, kps_xh, kms_xh;
};

__device__ __forceinline__ EColumn e_column(const StepParams& p, int j, int k) {
  EColumn c;
  c.f0 = in_runs(p.fuD[0], k); c.f2 = in_runs(p.fuD[2], j);
  c.w1 = in_runs(p.fwE[1], j); c.w2 = in_runs(p.fwE[2], k);
  c.kms_y = ldgf(p.kms[kInteger][1], j); c.sinv_y = ldgf(p.sinv[kInteger][1], j);
  c.kps_yh = ldgf(p.kps[kHalf][1], j); c.kms_yh = ldgf(p.kms[kHalf][1], j);
  c.kms_z = ldgf(p.kms[kInteger][2], k); c.sinv_z = ldgf(p.sinv[kInteger][2], k);
  c.kps_zh = ldgf(p.kps[kHalf][2], k); c.kms_zh = ldgf(p.kms[kHalf][2], k);
  return c;
}

__device__ __forceinline__ EPlane e_plane(const StepParams& p, int i) {
  EPlane c = {};
  c.f1 = in_runs(p.fuD[1], i); c.w0 = in_runs(p.fwE[0], i);
  return c;
}

// The plane's coefficients, needed only on the PML path.
__device__ __forceinline__ void e_plane_coefficients(const StepParams& p, int i, EPlane& c) {
  c.kms_x = ldgf(p.kms[kInteger][0], i); c.sinv_x = ldgf(p.sinv[kInteger][0], i);
  c.kps_xh = ldgf(p.kps[kHalf][0], i); c.kms_xh = ldgf(p.kms[kHalf][0], i);
}

// D from its curls, the source deposit, zero_metal_D, E (update_E) and P (update_P)
// for one cell at offset c, for a warp that may touch the x (SX), y (SY) and z (SZ)
// memberships (x: Dx own, Dy dsigu, Dz dsig; y: Dx dsig, Dy own, Dz dsigu; z: Dx dsigu,
// Dy dsig, Dz own). <false, false, false> is the plain update.
// Every auxiliary word an E cell reads (split-field fu of D and the old E on the
// own-axis membership), loaded from the flags alone with the field loads. f_w of E is
// not among them: its old word is recomputed from the old D (see e_cell_v).
struct EAux {
  float u[3], e[3];
};

__device__ __forceinline__ void e_aux_load(const StepParams& p, const EColumn& col, const EPlane& pl, int c,
                                           EAux& a) {
  const bool sf[3] = {col.f0, pl.f1, col.f2};
  const bool sw[3] = {pl.w0, col.w1, col.w2};
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    a.u[q] = sf[q] ? p.fuD[q].data[c] : 0.f;
    a.e[q] = sw[q] ? p.E[q][c] : 0.f;
  }
}

// Prefetch into L2 the auxiliary words a thread's cells of planes [i0, i1) will read
// (the PML counterpart of prefetch_planes), from the membership flags alone.
__device__ __forceinline__ void h_aux_prefetch(const StepParams& p, const HColumn& col, int c, int i0, int i1,
                                               int sx) {
  for (int i = i0; i < i1; ++i, c += sx) {
    const bool b[3] = {in_runs(p.B[0], i), col.b1, col.b2};
    const bool f[3] = {col.f0, in_runs(p.fuB[1], i), col.f2};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      if (b[q]) l2_prefetch(p.B[q].data + c);
      if (f[q]) l2_prefetch(p.fuB[q].data + c);
    }
  }
}

__device__ __forceinline__ void e_aux_prefetch(const StepParams& p, const EColumn& col, int c, int i0, int i1,
                                               int sx) {
  for (int i = i0; i < i1; ++i, c += sx) {
    const bool f[3] = {col.f0, in_runs(p.fuD[1], i), col.f2};
    const bool w[3] = {in_runs(p.fwE[0], i), col.w1, col.w2};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      if (f[q]) l2_prefetch(p.fuD[q].data + c);
      if (w[q]) l2_prefetch(p.E[q] + c);
    }
  }
}

template <bool SX, bool SY, bool SZ, bool COND = false>
__device__ __forceinline__ void e_cell_v(const StepParams& p, const EColumn& col, const EPlane& pl,
                                         int parity, int i, int j, int k, int c, float cx,
                                         float cy, float cz, float d[3], const float inv[3],
                                         const double* words, const EAux& a,
                                         const mgb_conductivity* cp = nullptr) {
  const bool wx = p.met[0] && i == 0, wy = p.met[1] && j == 0, wz = p.met[2] && k == 0;
  if (wy || wz) cx = 0.f;
  if (wx || wz) cy = 0.f;
  if (wx || wy) cz = 0.f;
  const bool sf0 = SZ && col.f0, sf1 = SX && pl.f1, sf2 = SY && col.f2;
  const bool sw0 = SX && pl.w0, sw1 = SY && col.w1, sw2 = SZ && col.w2;
  // The cell's auxiliary words (loaded by the caller, before any store).
  const float u0 = a.u[0], u1 = a.u[1], u2 = a.u[2];
  const float e0 = a.e[0], e1 = a.e[1], e2 = a.e[2];
  const bool in_box = p.npoles > 0 && i >= p.pbox[0] && i < p.pbox[1] && j >= p.pbox[2] &&
                      j < p.pbox[3] && k >= p.pbox[4] && k < p.pbox[5];
  long long pb = 0;
  if (in_box) {
    const int bny = p.pbox[3] - p.pbox[2], bnz = p.pbox[5] - p.pbox[4];
    pb = ((long long)(i - p.pbox[0]) * bny + (j - p.pbox[2])) * bnz + (k - p.pbox[4]);
  }
  // f_w of E: MEEP's update_E stores w = chi1inv (D - sum of P) in it on the own-axis
  // membership, so its old word is that expression of the old D (this cell's stored D)
  // and of the polarization the previous step subtracted (the buffer this step writes
  // P' over), in the same order of operations: recomputed here instead of stored.
  float fw[3] = {0.f, 0.f, 0.f};
  if (sw0 || sw1 || sw2) {
    fw[0] = d[0]; fw[1] = d[1]; fw[2] = d[2];
    if (in_box)
      for (int m = 0; m < p.npoles; ++m) {
        const mgb_pole& pole = p.poles[m];
#pragma unroll
        for (int q = 0; q < 3; ++q)
          if (pole.sigma[q] != nullptr) fw[q] = fw[q] - (parity ? pole.p[q][0] : pole.p[q][1])[pb];
      }
    fw[0] = inv[0] * fw[0];
    fw[1] = inv[1] * fw[1];
    fw[2] = inv[2] * fw[2];
  }
  const float fw0 = fw[0], fw1 = fw[1], fw2 = fw[2];
  // Dx: dsig y, dsigu z; Dy: dsig z, dsigu x; Dz: dsig x, dsigu y.
  float n0 = 0.f, n1 = 0.f, n2 = 0.f;
  if (COND) {
    // dsig of each component = the dsigu membership of the component two after it
    constexpr bool P = SX || SY || SZ;
    d[0] = cond_curl<P>(*cp, 1, 0, i, j, k, c, d[0], cx, col.f2, sf0, u0, col.kms_y, col.sinv_y, col.kms_z, col.sinv_z, n0);
    d[1] = cond_curl<P>(*cp, 1, 1, i, j, k, c, d[1], cy, col.f0, sf1, u1, col.kms_z, col.sinv_z, pl.kms_x, pl.sinv_x, n1);
    d[2] = cond_curl<P>(*cp, 1, 2, i, j, k, c, d[2], cz, pl.f1, sf2, u2, pl.kms_x, pl.sinv_x, col.kms_y, col.sinv_y, n2);
  } else {
    d[0] = curl_form<SY, SZ>(d[0], cx, sf0, u0, col.kms_y, col.sinv_y, col.kms_z, col.sinv_z, n0);
    d[1] = curl_form<SZ, SX>(d[1], cy, sf1, u1, col.kms_z, col.sinv_z, pl.kms_x, pl.sinv_x, n1);
    d[2] = curl_form<SX, SY>(d[2], cz, sf2, u2, pl.kms_x, pl.sinv_x, col.kms_y, col.sinv_y, n2);
  }
  // Electric sources at t + dt/2: f = float(double(f) - A), point by point in order.
  if (p.nsrc > p.nsrc_h && i >= p.src_box[0] && i < p.src_box[1] && j >= p.src_box[2] &&
      j < p.src_box[3] && k >= p.src_box[4] && k < p.src_box[5]) {
    for (int s = 0; s < p.nsrc - p.nsrc_h; ++s) {
      if (p.src_cell[s] != c) continue;
      const int q = p.src_comp[s];
      const double w = words[s];
      if (q == 0) d[0] = __double2float_rn(__dsub_rn((double)d[0], w));
      else if (q == 1) d[1] = __double2float_rn(__dsub_rn((double)d[1], w));
      else d[2] = __double2float_rn(__dsub_rn((double)d[2], w));
    }
  }
  // zero_metal_D: shift 0 on both transverse axes.
  if (wy || wz) d[0] = 0.f;
  if (wx || wz) d[1] = 0.f;
  if (wx || wy) d[2] = 0.f;
  float w[3] = {d[0], d[1], d[2]};
  if (in_box) {
    for (int m = 0; m < p.npoles; ++m) {
      const mgb_pole& pole = p.poles[m];
#pragma unroll
      for (int q = 0; q < 3; ++q)
        if (pole.sigma[q] != nullptr) w[q] = w[q] - (parity ? pole.p[q][1] : pole.p[q][0])[pb];
    }
  }
  w[0] = inv[0] * w[0];
  w[1] = inv[1] * w[1];
  w[2] = inv[2] * w[2];
  float e[3] = {w[0], w[1], w[2]};
  if (sw0) e[0] = e0 + (pl.kps_xh * w[0] - pl.kms_xh * fw0);
  if (sw1) e[1] = e1 + (col.kps_yh * w[1] - col.kms_yh * fw1);
  if (sw2) e[2] = e2 + (col.kps_zh * w[2] - col.kms_zh * fw2);
  if (sf0) p.fuD[0].data[c] = n0;
  if (sf1) p.fuD[1].data[c] = n1;
  if (sf2) p.fuD[2].data[c] = n2;
  p.D[0][c] = d[0];
  p.D[1][c] = d[1];
  p.D[2][c] = d[2];
  p.E[0][c] = e[0];
  p.E[1][c] = e[1];
  p.E[2][c] = e[2];
  const bool bad = !isfinite(e[0]) || !isfinite(e[1]) || !isfinite(e[2]);
  if (in_box) {
    // update_P: P' = g1inv*(((P*A) - (g1*Pp)) + (w0dt2*(s*W))), written over Pp.
    for (int m = 0; m < p.npoles; ++m) {
      const mgb_pole& pole = p.poles[m];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        if (pole.sigma[q] == nullptr) continue;
        const float* cur = parity ? pole.p[q][1] : pole.p[q][0];
        float* prv = parity ? pole.p[q][0] : pole.p[q][1];
        const float pc = cur[pb];
        const float pp = prv[pb];
        const float s = __ldg(pole.sigma[q] + pb);
        const float drive = pole.omega0dtsqr * (s * w[q]);
        prv[pb] = pole.gamma1inv * ((pc * pole.two_minus_od - pole.gamma1 * pp) + drive);
      }
    }
  }
  if (bad && p.status != nullptr) atomicOr(p.status, 1);
}

template <bool PML, bool COND = false, int AX = -1>
__device__ __forceinline__ void e_cell(const StepParams& p, const EColumn& col, const EPlane& pl,
                                       int axes, int parity, int i, int j, int k, int c, float cx,
                                       float cy, float cz, float d[3], const float inv[3],
                                       const double* words, const EAux& a,
                                       const mgb_conductivity* cp = nullptr) {
  if (COND) {
    // a lossy run: the variant of the CTA's axes, or the general one
    constexpr bool X = AX < 0 || (AX & 1), Y = AX < 0 || (AX & 2), Z = AX < 0 || (AX & 4);
    if (PML) e_cell_v<X, Y, Z, true>(p, col, pl, parity, i, j, k, c, cx, cy, cz, d, inv, words, a, cp);
    else e_cell_v<false, false, false, true>(p, col, pl, parity, i, j, k, c, cx, cy, cz, d, inv, words, a, cp);
    return;
  }
  if (!PML) axes = 0;
  switch (axes) {
    case 0: e_cell_v<false, false, false>(p, col, pl, parity, i, j, k, c, cx, cy, cz, d, inv, words, a); break;
    case 1: e_cell_v<true, false, false>(p, col, pl, parity, i, j, k, c, cx, cy, cz, d, inv, words, a); break;
    case 2: e_cell_v<false, true, false>(p, col, pl, parity, i, j, k, c, cx, cy, cz, d, inv, words, a); break;
    case 3: e_cell_v<true, true, false>(p, col, pl, parity, i, j, k, c, cx, cy, cz, d, inv, words, a); break;
    case 4: e_cell_v<false, false, true>(p, col, pl, parity, i, j, k, c, cx, cy, cz, d, inv, words, a); break;
    case 5: e_cell_v<true, false, true>(p, col, pl, parity, i, j, k, c, cx, cy, cz, d, inv, words, a); break;
    case 6: e_cell_v<false, true, true>(p, col, pl, parity, i, j, k, c, cx, cy, cz, d, inv, words, a); break;
    default: e_cell_v<true, true, true>(p, col, pl, parity, i, j, k, c, cx, cy, cz, d, inv, words, a); break;
  }
}

// Whether the next (previous) lane of the warp holds this thread's +z (-z) neighbour in
// the same block row: the block's rows are blockDim.x consecutive z cells, a warp holds
// one or more whole rows or 32 cells of one row.
__device__ __forceinline__ int lane_id() { return (int)((threadIdx.x + blockDim.x * threadIdx.y) & 31); }
__device__ __forceinline__ bool next_lane_has_z(int k, int nz) {
  return lane_id() != 31 && threadIdx.x + 1 < blockDim.x && k + 1 < nz;
}
__device__ __forceinline__ bool prev_lane_has_z() { return lane_id() != 0 && threadIdx.x > 0; }

// The axes (bit 0 x, 1 y, 2 z) along which a CTA's cells [i0, i1) x [j0, j0 + by) x
// [k0, k0 + bz) reach some membership: outside the range of the box no membership
// reaches (StepParams.inner) some auxiliary's run may hold a cell; inside it none does,
// so every coefficient of that axis is exactly 1 for the whole CTA. 0: the CTA steps the
// plain update, word for word.
// Whether a CTA holds index 0 of a Bloch-phased axis (its cells read across the face).
__device__ __forceinline__ bool cta_bloch(const StepParams& p, int i0, int j0, int k0) {
  return p.bloch && (((p.bloch & 1) && i0 == 0) || ((p.bloch & 2) && j0 == 0) || ((p.bloch & 4) && k0 == 0));
}

// Whether a CTA's cells reach the bounding box of the magnetic source points.
__device__ __forceinline__ bool cta_msrc(const StepParams& p, int i0, int i1, int j0, int by, int k0, int bz) {
  return p.nsrc_h > 0 && i0 < p.src_box_h[1] && i1 > p.src_box_h[0] && j0 < p.src_box_h[3] &&
         j0 + by > p.src_box_h[2] && k0 < p.src_box_h[5] && k0 + bz > p.src_box_h[4];
}

__device__ __forceinline__ int cta_axes(const StepParams& p, int i0, int i1, int j0, int by, int k0, int bz) {
  return ((i0 >= p.inner[0] && i1 <= p.inner[1]) ? 0 : 1) |
         ((j0 >= p.inner[2] && j0 + by <= p.inner[3]) ? 0 : 2) |
         ((k0 >= p.inner[4] && k0 + bz <= p.inner[5]) ? 0 : 4);
}

// Dispatch a march on the CTA's axes: MARCH(AXV, PMLV) expands to one call.
#define MGB_AXES_SWITCH(AXES, MARCH)           \
  switch (AXES) {                              \
    case 0: MARCH(-1, false); break;           \
    case 1: MARCH(1, true); break;             \
    case 2: MARCH(2, true); break;             \
    case 3: MARCH(3, true); break;             \
    case 4: MARCH(4, true); break;             \
    case 5: MARCH(5, true); break;             \
    case 6: MARCH(6, true); break;             \
    default: MARCH(7, true); break;            \
  }

// ------------------------------------------------------------------------------------
// Generic kernels: plain loads, one thread per (y, z) column marching over x.
// One thread's column (j, k) of the H half over planes [i0, i1).
template <bool PML, bool COND = false, int AX = -1, bool MSRC = false, bool BLOCH = false, bool RED = false>
__device__ __forceinline__ void h_march(const StepParams& p, int j, int k, int i0, int i1,
                                        int first_step, const mgb_conductivity* cp = nullptr) {
  const int sx = p.ny * p.nz;
  const int sy = p.nz;
  const float* Ex = p.E[0];
  const float* Ey = p.E[1];
  const float* Ez = p.E[2];
  const bool ytop = (j + 1 == p.ny), ztop = (k + 1 == p.nz);
  const bool ywall = ytop && p.met[1], zwall = ztop && p.met[2];
  const int oy = ytop ? -(p.ny - 1) * sy : sy;
  const int oz = ztop ? -(p.nz - 1) : 1;
  const int col = j * sy + k;
  int c = i0 * sx + col;
  if (p.l2pf) {
    const float* vols[6] = {Ex, Ey, Ez, p.H[0], p.H[1], p.H[2]};
    prefetch_planes(vols, 6, c, sx, i1 - i0);
  }
  HColumn hcol = {};
  int col_axes = 0;  // bit 1: the warp touches the y memberships, bit 2: the z ones
  if (PML) {
    hcol = h_column(p, j, k);
    if (AX < 0) {
      const unsigned lanes = __activemask();
      col_axes = (__any_sync(lanes, hcol.f2 || hcol.b1) ? 2 : 0) |
                 (__any_sync(lanes, hcol.f0 || hcol.b2) ? 4 : 0);
    }
    if (p.l2pf) h_aux_prefetch(p, hcol, c, i0, i1, sx);
  }
  float ey = Ey[c];
  float ez = Ez[c];
  for (int i = i0; i < i1; ++i, c += sx) {
    HPlane pl = {};
    int axes = 0;
    if (PML) {
      pl = h_plane(p, i);
      axes = AX >= 0 ? AX : COND ? 7 : col_axes | ((pl.f1 || pl.b0) ? 1 : 0);
      if (h_needs_plane(axes)) h_plane_coefficients(p, i, pl);
    }
    const float ex = Ex[c];
    float ey_xp, ez_xp;
    if (i + 1 < p.nx) {
      ey_xp = Ey[c + sx];
      ez_xp = Ez[c + sx];
    } else if (p.met[0]) {
      ey_xp = 0.f;
      ez_xp = 0.f;
    } else {
      ey_xp = Ey[col];
      ez_xp = Ez[col];
    }
    const float ez_yp = ywall ? 0.f : Ez[c + oy];
    const float ex_yp = ywall ? 0.f : Ex[c + oy];
    const float ey_zp = zwall ? 0.f : Ey[c + oz];
    const float ex_zp = zwall ? 0.f : Ex[c + oz];
    const float h_old[3] = {p.H[0][c], p.H[1][c], p.H[2][c]};
    HAux ax = {};
    if (PML && axes != 0) h_aux_load(p, hcol, pl, c, ax);
    // MEEP's association ((g1s - g1) + g2) - g2s, then the dtdx scale.
    // the same-index curl operands: on a Bloch-phased axis the word below the window
    // at index 0 (B's forward curl reads E at the low wall: conj(eikna) times the stored
    // top word, both parts)
    float gx1 = ez, gx2 = ey, gy1 = ex, gy2 = ez, gz1 = ey, gz2 = ex;
    if (BLOCH) {
      if (j == 0) { gx1 = bloch_word(p, 1, true, ez, p.pE[2], c); gz2 = bloch_word(p, 1, true, ex, p.pE[0], c); }
      if (k == 0) { gx2 = bloch_word(p, 2, true, ey, p.pE[1], c); gy1 = bloch_word(p, 2, true, ex, p.pE[0], c); }
      if (i == 0) { gy2 = bloch_word(p, 0, true, ez, p.pE[2], c); gz1 = bloch_word(p, 0, true, ey, p.pE[1], c); }
    }
    const float cx = curl_term<RED>(p, ez_yp, gx1, gx2, ey_zp, 1, 2);
    const float cy = curl_term<RED>(p, ex_zp, gy1, gy2, ez_xp, 2, 0);
    const float cz = curl_term<RED>(p, ey_xp, gz1, gz2, ex_yp, 0, 1);
    float h_new[3];
    h_cell<PML, COND, AX, MSRC>(p, hcol, pl, axes, first_step, i, j, k, c, cx, cy, cz, h_old, ax, h_new, cp);
    p.H[0][c] = h_new[0];
    p.H[1][c] = h_new[1];
    p.H[2][c] = h_new[2];
    ey = ey_xp;
    ez = ez_xp;
  }
}

// One thread's column (j, k) of the E half over planes [i0, i1).
template <bool PML, bool COND = false, int AX = -1, bool BLOCH = false, bool RED = false>
__device__ __forceinline__ void e_march(const StepParams& p, int j, int k, int i0, int i1,
                                        int parity, const double* words,
                                        const mgb_conductivity* cp = nullptr) {
  const int sx = p.ny * p.nz;
  const int sy = p.nz;
  const float* Hx = p.H[0];
  const float* Hy = p.H[1];
  const float* Hz = p.H[2];
  const int jm = j == 0 ? (p.met[1] ? -1 : p.ny - 1) : j - 1;
  const int km = k == 0 ? (p.met[2] ? -1 : p.nz - 1) : k - 1;
  const int col = j * sy + k;
  int c = i0 * sx + col;
  if (p.l2pf) {
    const float* vols[7] = {Hx, Hy, Hz, p.D[0], p.D[1], p.D[2], p.inv_eps[0]};
    prefetch_planes(vols, p.inv_eps[1] == p.inv_eps[0] ? 7 : 6, c, sx, i1 - i0);
  }
  EColumn ecol = {};
  int col_axes = 0;  // bit 1: the warp touches the y memberships, bit 2: the z ones
  if (PML) {
    ecol = e_column(p, j, k);
    if (AX < 0) {
      const unsigned lanes = __activemask();
      col_axes = (__any_sync(lanes, ecol.f2 || ecol.w1) ? 2 : 0) |
                 (__any_sync(lanes, ecol.f0 || ecol.w2) ? 4 : 0);
    }
    if (p.l2pf) e_aux_prefetch(p, ecol, c, i0, i1, sx);
  }
  float hy_xm = 0.f, hz_xm = 0.f;
  {
    int im = i0 - 1;
    if (im < 0) im = p.met[0] ? -1 : p.nx - 1;
    if (im >= 0) {
      hy_xm = Hy[im * sx + col];
      hz_xm = Hz[im * sx + col];
    }
  }
  for (int i = i0; i < i1; ++i, c += sx) {
    EPlane pl = {};
    int axes = 0;
    if (PML) {
      pl = e_plane(p, i);
      axes = AX >= 0 ? AX : COND ? 7 : col_axes | ((pl.f1 || pl.w0) ? 1 : 0);
      if (axes & 1) e_plane_coefficients(p, i, pl);
    }
    const float hx = Hx[c], hy = Hy[c], hz = Hz[c];
    float hz_ym = 0.f, hx_ym = 0.f, hy_zm = 0.f, hx_zm = 0.f;
    if (jm >= 0) {
      const int cm = i * sx + jm * sy + k;
      hz_ym = Hz[cm];
      hx_ym = Hx[cm];
    }
    if (km >= 0) {
      const int cm = i * sx + j * sy + km;
      hy_zm = Hy[cm];
      hx_zm = Hx[cm];
    }
    float d[3] = {p.D[0][c], p.D[1][c], p.D[2][c]};
    const float inv[3] = {__ldg(p.inv_eps[0] + c), __ldg(p.inv_eps[1] + c), __ldg(p.inv_eps[2] + c)};
    EAux ax = {};
    if (PML && axes != 0) e_aux_load(p, ecol, pl, c, ax);
    // on a Bloch-phased axis D's backward curl at index 0 reads H above the window:
    // eikna times the stored word, both parts
    float gx1 = hz, gx2 = hy, gy1 = hx, gy2 = hz, gz1 = hy, gz2 = hx;
    if (BLOCH) {
      if (j == 0) { gx1 = bloch_word(p, 1, false, hz, p.pH[2], c); gz2 = bloch_word(p, 1, false, hx, p.pH[0], c); }
      if (k == 0) { gx2 = bloch_word(p, 2, false, hy, p.pH[1], c); gy1 = bloch_word(p, 2, false, hx, p.pH[0], c); }
      if (i == 0) { gy2 = bloch_word(p, 0, false, hz, p.pH[2], c); gz1 = bloch_word(p, 0, false, hy, p.pH[1], c); }
    }
    const float cx = curl_term<RED>(p, hz_ym, gx1, gx2, hy_zm, 1, 2);
    const float cy = curl_term<RED>(p, hx_zm, gy1, gy2, hz_xm, 2, 0);
    const float cz = curl_term<RED>(p, hy_xm, gz1, gz2, hx_ym, 0, 1);
    e_cell<PML, COND, AX>(p, ecol, pl, axes, parity, i, j, k, c, cx, cy, cz, d, inv, words, ax, cp);
    hy_xm = hy;
    hz_xm = hz;
  }
}

// Prefetching marches: the same cell updates, with every field load of plane i + 1
// issued before plane i is computed and stored, so each thread keeps two planes of loads
// in flight (the loads of a plane do not depend on the stores of the one before: other
// cells, or the thread's own cell read before it is written). The z neighbours held by
// the adjacent lane of the same row come by shuffle instead of a load (with their 64
// registers these marches can afford it; at the generic marches' 48 it spilled).
struct HLoads {
  float ex, ey_xp, ez_xp, ez_yp, ex_yp, ey_zp, ex_zp, h[3];
};

__device__ __forceinline__ void h_loads(const StepParams& p, HLoads& L, int i, int c, int col, int sx,
                                        int oy, int oz, bool ywall, bool zwall, bool z_from_lane) {
  L.ex = p.E[0][c];
  if (i + 1 < p.nx) {
    L.ey_xp = p.E[1][c + sx];
    L.ez_xp = p.E[2][c + sx];
  } else if (p.met[0]) {
    L.ey_xp = 0.f;
    L.ez_xp = 0.f;
  } else {
    L.ey_xp = p.E[1][col];
    L.ez_xp = p.E[2][col];
  }
  L.ez_yp = ywall ? 0.f : p.E[2][c + oy];
  L.ex_yp = ywall ? 0.f : p.E[0][c + oy];
  // +z neighbours: loaded only by lanes whose next lane does not hold them
  L.ey_zp = (zwall || z_from_lane) ? 0.f : p.E[1][c + oz];
  L.ex_zp = (zwall || z_from_lane) ? 0.f : p.E[0][c + oz];
  L.h[0] = p.H[0][c];
  L.h[1] = p.H[1][c];
  L.h[2] = p.H[2][c];
}

template <bool PML, int AX = -1, bool MSRC = false, bool RED = false>
__device__ __forceinline__ void h_march_pf(const StepParams& p, int j, int k, int i0, int i1,
                                           int first_step) {
  const int sx = p.ny * p.nz;
  const int sy = p.nz;
  const bool ytop = (j + 1 == p.ny), ztop = (k + 1 == p.nz);
  const bool ywall = ytop && p.met[1], zwall = ztop && p.met[2];
  const int oy = ytop ? -(p.ny - 1) * sy : sy;
  const int oz = ztop ? -(p.nz - 1) : 1;
  const int col = j * sy + k;
  int c = i0 * sx + col;
  if (p.l2pf) {
    const float* vols[6] = {p.E[0], p.E[1], p.E[2], p.H[0], p.H[1], p.H[2]};
    prefetch_planes(vols, 6, c, sx, i1 - i0);
  }
  HColumn hcol = {};
  int col_axes = 0;
  if (PML) {
    hcol = h_column(p, j, k);
    if (AX < 0) {
      const unsigned lanes = __activemask();
      col_axes = (__any_sync(lanes, hcol.f2 || hcol.b1) ? 2 : 0) |
                 (__any_sync(lanes, hcol.f0 || hcol.b2) ? 4 : 0);
    }
    if (p.l2pf) h_aux_prefetch(p, hcol, c, i0, i1, sx);
  }
  float ey = p.E[1][c];
  float ez = p.E[2][c];
  const unsigned zlanes = __activemask();
  const bool z_from_lane = next_lane_has_z(k, p.nz);
  HLoads cur;
  h_loads(p, cur, i0, c, col, sx, oy, oz, ywall, zwall, z_from_lane);
  for (int i = i0; i < i1; ++i, c += sx) {
    HLoads nxt;
    if (i + 1 < i1) h_loads(p, nxt, i + 1, c + sx, col, sx, oy, oz, ywall, zwall, z_from_lane);
    {
      const float ey_up = __shfl_down_sync(zlanes, ey, 1);
      const float ex_up = __shfl_down_sync(zlanes, cur.ex, 1);
      if (z_from_lane && !zwall) {
        cur.ey_zp = ey_up;
        cur.ex_zp = ex_up;
      }
    }
    HPlane pl = {};
    int axes = 0;
    if (PML) {
      pl = h_plane(p, i);
      axes = AX >= 0 ? AX : col_axes | ((pl.f1 || pl.b0) ? 1 : 0);
      if (h_needs_plane(axes)) h_plane_coefficients(p, i, pl);
    }
    HAux ax = {};
    if (PML && axes != 0) h_aux_load(p, hcol, pl, c, ax);
    const float cx = curl_term<RED>(p, cur.ez_yp, ez, ey, cur.ey_zp, 1, 2);
    const float cy = curl_term<RED>(p, cur.ex_zp, cur.ex, ez, cur.ez_xp, 2, 0);
    const float cz = curl_term<RED>(p, cur.ey_xp, ey, cur.ex, cur.ex_yp, 0, 1);
    float h_new[3];
    h_cell<PML, false, AX, MSRC>(p, hcol, pl, axes, first_step, i, j, k, c, cx, cy, cz, cur.h, ax, h_new);
    p.H[0][c] = h_new[0];
    p.H[1][c] = h_new[1];
    p.H[2][c] = h_new[2];
    ey = cur.ey_xp;
    ez = cur.ez_xp;
    cur = nxt;
  }
}

struct ELoads {
  float hx, hy, hz, hz_ym, hx_ym, hy_zm, hx_zm, d[3], inv[3];
};

__device__ __forceinline__ void e_loads(const StepParams& p, ELoads& L, int i, int c, int j, int k, int jm,
                                        int km, int sx, int sy) {
  L.hx = p.H[0][c];
  L.hy = p.H[1][c];
  L.hz = p.H[2][c];
  L.hz_ym = L.hx_ym = L.hy_zm = L.hx_zm = 0.f;
  if (jm >= 0) {
    const int cm = i * sx + jm * sy + k;
    L.hz_ym = p.H[2][cm];
    L.hx_ym = p.H[0][cm];
  }
  // -z neighbours: loaded only where the previous lane does not hold them
  if (km >= 0 && !prev_lane_has_z()) {
    const int cm = i * sx + j * sy + km;
    L.hy_zm = p.H[1][cm];
    L.hx_zm = p.H[0][cm];
  }
  L.d[0] = p.D[0][c];
  L.d[1] = p.D[1][c];
  L.d[2] = p.D[2][c];
  L.inv[0] = __ldg(p.inv_eps[0] + c);
  L.inv[1] = __ldg(p.inv_eps[1] + c);
  L.inv[2] = __ldg(p.inv_eps[2] + c);
}

template <bool PML, int AX = -1, bool RED = false>
__device__ __forceinline__ void e_march_pf(const StepParams& p, int j, int k, int i0, int i1,
                                           int parity, const double* words) {
  const int sx = p.ny * p.nz;
  const int sy = p.nz;
  const int jm = j == 0 ? (p.met[1] ? -1 : p.ny - 1) : j - 1;
  const int km = k == 0 ? (p.met[2] ? -1 : p.nz - 1) : k - 1;
  const int col = j * sy + k;
  int c = i0 * sx + col;
  if (p.l2pf) {
    const float* vols[7] = {p.H[0], p.H[1], p.H[2], p.D[0], p.D[1], p.D[2], p.inv_eps[0]};
    prefetch_planes(vols, p.inv_eps[1] == p.inv_eps[0] ? 7 : 6, c, sx, i1 - i0);
  }
  EColumn ecol = {};
  int col_axes = 0;
  if (PML) {
    ecol = e_column(p, j, k);
    if (AX < 0) {
      const unsigned lanes = __activemask();
      col_axes = (__any_sync(lanes, ecol.f2 || ecol.w1) ? 2 : 0) |
                 (__any_sync(lanes, ecol.f0 || ecol.w2) ? 4 : 0);
    }
    if (p.l2pf) e_aux_prefetch(p, ecol, c, i0, i1, sx);
  }
  float hy_xm = 0.f, hz_xm = 0.f;
  {
    int im = i0 - 1;
    if (im < 0) im = p.met[0] ? -1 : p.nx - 1;
    if (im >= 0) {
      hy_xm = p.H[1][im * sx + col];
      hz_xm = p.H[2][im * sx + col];
    }
  }
  const unsigned zlanes = __activemask();
  ELoads cur;
  e_loads(p, cur, i0, c, j, k, jm, km, sx, sy);
  for (int i = i0; i < i1; ++i, c += sx) {
    ELoads nxt;
    if (i + 1 < i1) e_loads(p, nxt, i + 1, c + sx, j, k, jm, km, sx, sy);
    {
      const float hy_dn = __shfl_up_sync(zlanes, cur.hy, 1);
      const float hx_dn = __shfl_up_sync(zlanes, cur.hx, 1);
      if (prev_lane_has_z()) {
        cur.hy_zm = hy_dn;
        cur.hx_zm = hx_dn;
      }
    }
    EPlane pl = {};
    int axes = 0;
    if (PML) {
      pl = e_plane(p, i);
      axes = AX >= 0 ? AX : col_axes | ((pl.f1 || pl.w0) ? 1 : 0);
      if (axes & 1) e_plane_coefficients(p, i, pl);
    }
    EAux ax = {};
    if (PML && axes != 0) e_aux_load(p, ecol, pl, c, ax);
    const float cx = curl_term<RED>(p, cur.hz_ym, cur.hz, cur.hy, cur.hy_zm, 1, 2);
    const float cy = curl_term<RED>(p, cur.hx_zm, cur.hx, cur.hz, hz_xm, 2, 0);
    const float cz = curl_term<RED>(p, hy_xm, cur.hy, cur.hx, cur.hx_ym, 0, 1);
    e_cell<PML, false, AX>(p, ecol, pl, axes, parity, i, j, k, c, cx, cy, cz, cur.d, cur.inv, words, ax);
    hy_xm = cur.hy;
    hz_xm = cur.hz;
    cur = nxt;
  }
}

}  // namespace mgbstep
