// meepgb.cu — GB300 (sm_103a) FDTD stepping kernels and the C ABI of libmeepgb.so.
//
// One step is two fused kernels:
//   h_half: MEEP's step_B (curl E with the split-field UPML), zero_metal_B and
//           update_H (own-axis constitutive accumulation, H aliased to B outside it);
//   e_half: step_D, the electric source deposit in double, zero_metal_D, update_E
//           (chi1inv of D minus every polarization, own-axis accumulation) and update_P
//           (Lorentz/Drude ADE), all on registers of one cell.
// followed on decimated steps by dft_accumulate for every monitor.
//
// Arithmetic follows the reference array path operation for operation (meep_gpu/
// stepping.py: _curl_from_operands :2265, _apply_pml_update :2629,
// _apply_dsig_only_update :2662, _apply_constitutive_pml :2991, separate_h_from_b
// :2789, _mask_non_owned_cells :2589, _zero_metal :3135; dispersion.py
// PolarizationState.update :689; sources.py _deposit :1357). The file is compiled
// with -fmad=false so no multiply-add is contracted, which keeps every float32 word
// equal to the reference's separately rounded operations.
//
// Work decomposition: a CTA covers a (BZ x BY) tile of (z, y) columns and marches
// along x over a chunk of planes; the x-neighbour a stencil needs (E at i+1 for the H
// half, H at i-1 for the E half) is carried in registers from the previous plane, and
// the y/z neighbours are re-read through L1. Each cell's word is read from HBM once
// per half step. PML auxiliaries live in compact slab arrays over the membership runs.

#include "meepgb.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>

namespace {

thread_local std::string g_error;

int fail(int code, const std::string& message) {
  g_error = message;
  return code;
}

// ------------------------------------------------------------------------------------
// Parameters passed by value (__grid_constant__) to the step kernels.
struct StepParams {
  int nx, ny, nz;
  int met[3];
  float dtdx;
  const float* kms[2][3];
  const float* sinv[2][3];
  const float* kps[2][3];
  float* E[3];
  float* D[3];
  float* B[3];
  const float* inv_eps[3];
  mgb_aux H[3], fwH[3], fwE[3], fuB[3], fuD[3];
  int npoles;
  int pbox[6];
  mgb_pole poles[MGB_MAX_POLES];
  int nsrc;
  const int64_t* src_cell;
  const int32_t* src_comp;
  int src_box[6];
  const double* src_words;  // row for the current step, [nsrc]
  int32_t* status;
};

struct DftParams {
  int nx, ny, nz;
  int met[3];
  int pml;
  const float* E[3];
  const float* B[3];
  mgb_aux H[3];
  mgb_monitor mon;
};

constexpr int kInteger = 0;
constexpr int kHalf = 1;

__device__ __forceinline__ int slab_row(const mgb_aux& a, int i) {
  if (i >= a.a0 && i < a.a1) return i - a.a0;
  if (i >= a.b0 && i < a.b1) return (a.a1 - a.a0) + (i - a.b0);
  return -1;
}

template <int AXIS>
__device__ __forceinline__ long long aux_index(const mgb_aux& a, int row, int i, int j, int k,
                                               int ny, int nz) {
  const int m = (a.a1 - a.a0) + (a.b1 - a.b0);
  if (AXIS == 0) return ((long long)row * ny + j) * nz + k;
  if (AXIS == 1) return ((long long)i * m + row) * nz + k;
  return ((long long)i * ny + j) * m + row;
}

// The split-field curl update of one B/D component (MEEP step_curl, both forms).
//   inside the dsigu membership: fu' = ((kms*fu) - curl)*sinv;
//                                f'  = (((kms_u*f) + fu') - fu)*sinv_u
//   elsewhere:                   f'  = ((kms*f) - curl)*sinv
template <int UAXIS>
__device__ __forceinline__ float curl_update(const StepParams& p, int lattice, int sig_axis,
                                             const mgb_aux& fu, float f, float curl, int i,
                                             int j, int k) {
  const int sig_at = sig_axis == 0 ? i : (sig_axis == 1 ? j : k);
  const int u_at = UAXIS == 0 ? i : (UAXIS == 1 ? j : k);
  const float kms = __ldg(p.kms[lattice][sig_axis] + sig_at);
  const float sinv = __ldg(p.sinv[lattice][sig_axis] + sig_at);
  const int row = slab_row(fu, u_at);
  if (row >= 0) {
    const long long a = aux_index<UAXIS>(fu, row, i, j, k, p.ny, p.nz);
    const float prev = fu.data[a];
    const float next = (kms * prev - curl) * sinv;
    fu.data[a] = next;
    const float kms_u = __ldg(p.kms[lattice][UAXIS] + u_at);
    const float sinv_u = __ldg(p.sinv[lattice][UAXIS] + u_at);
    return ((kms_u * f + next) - prev) * sinv_u;
  }
  return (kms * f - curl) * sinv;
}

// ------------------------------------------------------------------------------------
// H half: B -= curl E (split-field UPML), zero_metal_B, H from B.
template <bool PML>
__global__ void __launch_bounds__(256) h_half(const __grid_constant__ StepParams p,
                                              int first_step, int xchunk) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (k >= p.nz || j >= p.ny) return;
  const int i0 = blockIdx.z * xchunk;
  const int i1 = min(i0 + xchunk, p.nx);
  const long long sx = (long long)p.ny * p.nz;
  const long long sy = p.nz;
  const float* __restrict__ Ex = p.E[0];
  const float* __restrict__ Ey = p.E[1];
  const float* __restrict__ Ez = p.E[2];
  const float dtdx = p.dtdx;
  // Offsets of the +1 neighbours; a metallic far face reads the zero ghost instead.
  const bool ytop = (j + 1 == p.ny), ztop = (k + 1 == p.nz);
  const bool ywall = ytop && p.met[1], zwall = ztop && p.met[2];
  const long long oy = ytop ? -(long long)(p.ny - 1) * sy : sy;
  const long long oz = ztop ? -(long long)(p.nz - 1) : 1;
  const long long col = (long long)j * sy + k;
  long long c = (long long)i0 * sx + col;
  float ey = Ey[c];
  float ez = Ez[c];
  for (int i = i0; i < i1; ++i, c += sx) {
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
    // MEEP's association ((g1s - g1) + g2) - g2s, then the dtdx scale.
    float cx = dtdx * (((ez_yp - ez) + ey) - ey_zp);
    float cy = dtdx * (((ex_zp - ex) + ez) - ez_xp);
    float cz = dtdx * (((ey_xp - ey) + ex) - ex_yp);
    // Owned-cell masks: a shift-0 axis on a metallic wall does not step cell 0.
    if (p.met[0] && i == 0) cx = 0.f;
    if (p.met[1] && j == 0) cy = 0.f;
    if (p.met[2] && k == 0) cz = 0.f;
    float bx = p.B[0][c], by = p.B[1][c], bz = p.B[2][c];
    if (PML) {
      // Bx: dsig y, dsigu z; By: dsig z, dsigu x; Bz: dsig x, dsigu y (half lattice).
      bx = curl_update<2>(p, kHalf, 1, p.fuB[0], bx, cx, i, j, k);
      by = curl_update<0>(p, kHalf, 2, p.fuB[1], by, cy, i, j, k);
      bz = curl_update<1>(p, kHalf, 0, p.fuB[2], bz, cz, i, j, k);
    } else {
      bx = bx - cx;
      by = by - cy;
      bz = bz - cz;
    }
    // zero_metal_B: the component sits on the wall of every axis where its shift is 0.
    if (p.met[0] && i == 0) bx = 0.f;
    if (p.met[1] && j == 0) by = 0.f;
    if (p.met[2] && k == 0) bz = 0.f;
    p.B[0][c] = bx;
    p.B[1][c] = by;
    p.B[2][c] = bz;
    if (PML) {
      // update_H on the own-axis integer membership: fw' = B, H' = H + ((kps*B) - (kms*fw)).
      const float bs[3] = {bx, by, bz};
      const int at[3] = {i, j, k};
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const int row = slab_row(p.H[q], at[q]);
        if (row < 0) continue;
        long long a;
        if (q == 0) a = aux_index<0>(p.H[0], row, i, j, k, p.ny, p.nz);
        else if (q == 1) a = aux_index<1>(p.H[1], row, i, j, k, p.ny, p.nz);
        else a = aux_index<2>(p.H[2], row, i, j, k, p.ny, p.nz);
        const float fw_prev = first_step ? bs[q] : p.fwH[q].data[a];
        const float h_prev = first_step ? bs[q] : p.H[q].data[a];
        const float kps = __ldg(p.kps[kInteger][q] + at[q]);
        const float kms = __ldg(p.kms[kInteger][q] + at[q]);
        p.fwH[q].data[a] = bs[q];
        p.H[q].data[a] = h_prev + (kps * bs[q] - kms * fw_prev);
      }
    }
    ey = ey_xp;
    ez = ez_xp;
  }
}

// H component q at (i, j, k): the stored own-axis slab word, or B's word outside it.
template <bool PML, int Q>
__device__ __forceinline__ float read_h(const StepParams& p, long long c, int i, int j, int k) {
  if (PML) {
    const int at = Q == 0 ? i : (Q == 1 ? j : k);
    const int row = slab_row(p.H[Q], at);
    if (row >= 0) return p.H[Q].data[aux_index<Q>(p.H[Q], row, i, j, k, p.ny, p.nz)];
  }
  return p.B[Q][c];
}

// ------------------------------------------------------------------------------------
// E half: D += curl H (negated strides), source deposit, zero_metal_D, E, P.
template <bool PML>
__global__ void __launch_bounds__(256) e_half(const __grid_constant__ StepParams p, int parity,
                                              int xchunk) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (k >= p.nz || j >= p.ny) return;
  const int i0 = blockIdx.z * xchunk;
  const int i1 = min(i0 + xchunk, p.nx);
  const long long sx = (long long)p.ny * p.nz;
  const long long sy = p.nz;
  const float dtdx = p.dtdx;
  const bool ybot = (j == 0), zbot = (k == 0);
  const int jm = ybot ? (p.met[1] ? -1 : p.ny - 1) : j - 1;
  const int km = zbot ? (p.met[2] ? -1 : p.nz - 1) : k - 1;
  const long long col = (long long)j * sy + k;
  long long c = (long long)i0 * sx + col;
  // H at i0 - 1 (x-neighbour below) for Hy and Hz.
  float hy_xm = 0.f, hz_xm = 0.f;
  {
    int im = i0 - 1;
    if (im < 0) im = p.met[0] ? -1 : p.nx - 1;
    if (im >= 0) {
      const long long cm = (long long)im * sx + col;
      hy_xm = read_h<PML, 1>(p, cm, im, j, k);
      hz_xm = read_h<PML, 2>(p, cm, im, j, k);
    }
  }
  const bool src_cols = p.nsrc > 0 && j >= p.src_box[2] && j < p.src_box[3] &&
                        k >= p.src_box[4] && k < p.src_box[5];
  for (int i = i0; i < i1; ++i, c += sx) {
    const float hx = read_h<PML, 0>(p, c, i, j, k);
    const float hy = read_h<PML, 1>(p, c, i, j, k);
    const float hz = read_h<PML, 2>(p, c, i, j, k);
    float hz_ym = 0.f, hx_ym = 0.f, hy_zm = 0.f, hx_zm = 0.f;
    if (jm >= 0) {
      const long long cm = (long long)i * sx + (long long)jm * sy + k;
      hz_ym = read_h<PML, 2>(p, cm, i, jm, k);
      hx_ym = read_h<PML, 0>(p, cm, i, jm, k);
    }
    if (km >= 0) {
      const long long cm = (long long)i * sx + (long long)j * sy + km;
      hy_zm = read_h<PML, 1>(p, cm, i, j, km);
      hx_zm = read_h<PML, 0>(p, cm, i, j, km);
    }
    float cx = dtdx * (((hz_ym - hz) + hy) - hy_zm);
    float cy = dtdx * (((hx_zm - hx) + hz) - hz_xm);
    float cz = dtdx * (((hy_xm - hy) + hx) - hx_ym);
    const bool wx = p.met[0] && i == 0, wy = p.met[1] && j == 0, wz = p.met[2] && k == 0;
    if (wy || wz) cx = 0.f;
    if (wx || wz) cy = 0.f;
    if (wx || wy) cz = 0.f;
    float d[3] = {p.D[0][c], p.D[1][c], p.D[2][c]};
    if (PML) {
      // Dx: dsig y, dsigu z; Dy: dsig z, dsigu x; Dz: dsig x, dsigu y (integer lattice).
      d[0] = curl_update<2>(p, kInteger, 1, p.fuD[0], d[0], cx, i, j, k);
      d[1] = curl_update<0>(p, kInteger, 2, p.fuD[1], d[1], cy, i, j, k);
      d[2] = curl_update<1>(p, kInteger, 0, p.fuD[2], d[2], cz, i, j, k);
    } else {
      d[0] = d[0] - cx;
      d[1] = d[1] - cy;
      d[2] = d[2] - cz;
    }
    // Electric sources at t + dt/2: f = float(double(f) - A), point by point in order.
    if (src_cols && i >= p.src_box[0] && i < p.src_box[1]) {
      for (int s = 0; s < p.nsrc; ++s) {
        if (p.src_cell[s] != c) continue;
        const int q = p.src_comp[s];
        const double a = p.src_words[s];
        if (q == 0) d[0] = __double2float_rn(__dsub_rn((double)d[0], a));
        else if (q == 1) d[1] = __double2float_rn(__dsub_rn((double)d[1], a));
        else d[2] = __double2float_rn(__dsub_rn((double)d[2], a));
      }
    }
    // zero_metal_D.
    if (wy || wz) d[0] = 0.f;
    if (wx || wz) d[1] = 0.f;
    if (wx || wy) d[2] = 0.f;
    p.D[0][c] = d[0];
    p.D[1][c] = d[1];
    p.D[2][c] = d[2];
    // Polarization box position of this cell.
    const bool in_box = p.npoles > 0 && i >= p.pbox[0] && i < p.pbox[1] && j >= p.pbox[2] &&
                        j < p.pbox[3] && k >= p.pbox[4] && k < p.pbox[5];
    long long pb = 0;
    if (in_box) {
      const int bny = p.pbox[3] - p.pbox[2], bnz = p.pbox[5] - p.pbox[4];
      pb = ((long long)(i - p.pbox[0]) * bny + (j - p.pbox[2])) * bnz + (k - p.pbox[4]);
    }
    const int at[3] = {i, j, k};
    bool bad = false;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      float dmp = d[q];
      if (in_box) {
        for (int m = 0; m < p.npoles; ++m) {
          if (p.poles[m].sigma[q] != nullptr) dmp = dmp - p.poles[m].p[q][parity][pb];
        }
      }
      const float w = __ldg(p.inv_eps[q] + c) * dmp;
      float e = w;
      if (PML) {
        const int row = slab_row(p.fwE[q], at[q]);
        if (row >= 0) {
          long long a;
          if (q == 0) a = aux_index<0>(p.fwE[0], row, i, j, k, p.ny, p.nz);
          else if (q == 1) a = aux_index<1>(p.fwE[1], row, i, j, k, p.ny, p.nz);
          else a = aux_index<2>(p.fwE[2], row, i, j, k, p.ny, p.nz);
          const float fw_prev = p.fwE[q].data[a];
          p.fwE[q].data[a] = w;
          const float kps = __ldg(p.kps[kHalf][q] + at[q]);
          const float kms = __ldg(p.kms[kHalf][q] + at[q]);
          e = p.E[q][c] + (kps * w - kms * fw_prev);
        }
      }
      p.E[q][c] = e;
      bad |= !isfinite(e);
      if (in_box) {
        // update_P: P' = g1inv*(((P*A) - (g1*Pp)) + (w0dt2*(s*W))), written over Pp.
        for (int m = 0; m < p.npoles; ++m) {
          const mgb_pole& pole = p.poles[m];
          if (pole.sigma[q] == nullptr) continue;
          float* cur = pole.p[q][parity];
          float* prv = pole.p[q][parity ^ 1];
          const float pc = cur[pb];
          const float pp = prv[pb];
          const float s = __ldg(pole.sigma[q] + pb);
          const float drive = pole.omega0dtsqr * (s * w);
          prv[pb] = pole.gamma1inv * ((pc * pole.two_minus_od - pole.gamma1 * pp) + drive);
        }
      }
    }
    if (bad && p.status != nullptr) atomicOr(p.status, 1);
    hy_xm = hy;
    hz_xm = hz;
  }
}

// ------------------------------------------------------------------------------------
// DFT accumulation on one monitor: cell-centred samples times float64-formed phases.
template <bool PML, int Q>
__device__ __forceinline__ float read_h_dft(const DftParams& p, long long c, int i, int j,
                                            int k) {
  if (PML) {
    const int at = Q == 0 ? i : (Q == 1 ? j : k);
    const int row = slab_row(p.H[Q], at);
    if (row >= 0) return p.H[Q].data[aux_index<Q>(p.H[Q], row, i, j, k, p.ny, p.nz)];
  }
  return p.B[Q][c];
}

template <bool PML>
__device__ float field_at(const DftParams& p, int comp, int i, int j, int k) {
  // Past a face: metallic walls hold zero, periodic axes wrap.
  if (i >= p.nx) { if (p.met[0]) return 0.f; i -= p.nx; }
  if (j >= p.ny) { if (p.met[1]) return 0.f; j -= p.ny; }
  if (k >= p.nz) { if (p.met[2]) return 0.f; k -= p.nz; }
  const long long c = ((long long)i * p.ny + j) * p.nz + k;
  if (comp < 3) return p.E[comp][c];
  if (comp == 3) return read_h_dft<PML, 0>(p, c, i, j, k);
  if (comp == 4) return read_h_dft<PML, 1>(p, c, i, j, k);
  return read_h_dft<PML, 2>(p, c, i, j, k);
}

// Yee-to-centre average along every axis where the component's shift is 0, x then y
// then z, each 0.5*(f[i] + f[i+1]) in float32 (reference dft.py:352).
template <bool PML>
__device__ float centred(const DftParams& p, int comp, int i, int j, int k) {
  // Yee shifts: Ex (1,0,0) Ey (0,1,0) Ez (0,0,1) Hx (0,1,1) Hy (1,0,1) Hz (1,1,0).
  const int q = comp % 3;
  const bool electric = comp < 3;
  const bool ax = electric ? (q != 0) : (q == 0);
  const bool ay = electric ? (q != 1) : (q == 1);
  const bool az = electric ? (q != 2) : (q == 2);
  float v[2][2];
#pragma unroll
  for (int b = 0; b < 2; ++b) {
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      if ((a && !ay) || (b && !az)) { v[b][a] = 0.f; continue; }
      const float f0 = field_at<PML>(p, comp, i, j + a, k + b);
      v[b][a] = ax ? 0.5f * (f0 + field_at<PML>(p, comp, i + 1, j + a, k + b)) : f0;
    }
  }
  float r0 = ay ? 0.5f * (v[0][0] + v[0][1]) : v[0][0];
  if (!az) return r0;
  float r1 = ay ? 0.5f * (v[1][0] + v[1][1]) : v[1][0];
  return 0.5f * (r0 + r1);
}

template <bool PML>
__global__ void __launch_bounds__(256) dft_accumulate(const __grid_constant__ DftParams p,
                                                      long long step) {
  extern __shared__ float2 phase[];  // [0, nf): E phases, [nf, 2nf): H phases
  const mgb_monitor& m = p.mon;
  const int nf = m.nfreq;
  const double t_e = (double)step * m.dt;
  const double t_h = t_e - 0.5 * m.dt;
  for (int f = threadIdx.x; f < nf; f += blockDim.x) {
    const double w = m.omega[f];
    double s, co;
    sincos(t_e * w, &s, &co);
    phase[f] = make_float2((float)(co * m.scale), (float)(s * m.scale));
    sincos(t_h * w, &s, &co);
    phase[nf + f] = make_float2((float)(co * m.scale), (float)(s * m.scale));
  }
  __syncthreads();
  const int rx = m.region[1] - m.region[0], ry = m.region[3] - m.region[2],
            rz = m.region[5] - m.region[4];
  const long long cells = (long long)rx * ry * rz;
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= cells) return;
  const int rk = (int)(cell % rz);
  const int rj = (int)((cell / rz) % ry);
  const int ri = (int)(cell / ((long long)ry * rz));
  const int i = m.region[0] + ri, j = m.region[2] + rj, k = m.region[4] + rk;
  for (int q = 0; q < m.ncomp; ++q) {
    const int comp = m.comp[q];
    const float s = centred<PML>(p, comp, i, j, k);
    const float2* ph = comp < 3 ? phase : phase + nf;
    float* acc = m.acc + (long long)q * nf * 2 * cells + cell;
    for (int f = 0; f < nf; ++f) {
      float* re = acc + (long long)(2 * f) * cells;
      float* im = re + cells;
      *re = *re + ph[f].x * s;
      *im = *im + ph[f].y * s;
    }
  }
}

// Flux reduction, one block per frequency, float64 sums.
__global__ void __launch_bounds__(256) flux_reduce(const __grid_constant__ mgb_monitor m,
                                                   const float* __restrict__ weights,
                                                   double* __restrict__ out) {
  const int f = blockIdx.x;
  const long long cells = (long long)(m.region[1] - m.region[0]) * (m.region[3] - m.region[2]) *
                          (m.region[5] - m.region[4]);
  const long long plane = 2 * cells;
  const float* ea = m.acc + ((long long)0 * m.nfreq + f) * plane;
  const float* eb = m.acc + ((long long)1 * m.nfreq + f) * plane;
  const float* ha = m.acc + ((long long)2 * m.nfreq + f) * plane;
  const float* hb = m.acc + ((long long)3 * m.nfreq + f) * plane;
  double sum = 0.0;
  for (long long c = threadIdx.x; c < cells; c += blockDim.x) {
    const double w = weights[c];
    const double t1 = (double)ea[c] * hb[c] + (double)ea[cells + c] * hb[cells + c];
    const double t2 = (double)eb[c] * ha[c] + (double)eb[cells + c] * ha[cells + c];
    sum += w * (t1 - t2);
  }
  __shared__ double part[256];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[f] = part[0];
}

}  // namespace

// ======================================================================================
// C ABI
struct mgb_sim {
  mgb_sim_desc desc;
  StepParams step;
  const double* words = nullptr;
  long long words_first = 0;
  long long words_steps = 0;
  int block_z = 32;
  int block_y = 8;
  int xchunk = 16;
};

namespace {

bool aux_ok(const mgb_aux& a, int axis, int n, std::string* why, const char* name, int q) {
  if (a.data == nullptr || a.axis != axis || a.a0 < 0 || a.a0 > a.a1 || a.a1 > a.b0 ||
      a.b0 > a.b1 || a.b1 > n) {
    char buf[160];
    snprintf(buf, sizeof buf, "PML auxiliary %s[%d] is missing or its runs (%d,%d,%d,%d) on axis %d "
             "are not ordered inside 0..%d", name, q, a.a0, a.a1, a.b0, a.b1, a.axis, n);
    *why = buf;
    return false;
  }
  return true;
}

int launch_error(const char* what) {
  const cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) {
    return fail(MGB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(err));
  }
  return MGB_OK;
}

}  // namespace

extern "C" {

int mgb_abi_version(void) { return MGB_ABI_VERSION; }

int mgb_last_error(char* buf, size_t size) {
  if (buf == nullptr || size == 0) return MGB_ERR_ARGUMENT;
  const size_t n = g_error.size() < size - 1 ? g_error.size() : size - 1;
  memcpy(buf, g_error.data(), n);
  buf[n] = '\0';
  return MGB_OK;
}

int mgb_create(const mgb_sim_desc* desc, mgb_sim** out) {
  if (desc == nullptr || out == nullptr) return fail(MGB_ERR_ARGUMENT, "null descriptor or output");
  *out = nullptr;
  const mgb_sim_desc& d = *desc;
  if (d.abi_version != MGB_ABI_VERSION) {
    return fail(MGB_ERR_ARGUMENT, "descriptor ABI version " + std::to_string(d.abi_version) +
                                      " does not match the library's " +
                                      std::to_string(MGB_ABI_VERSION));
  }
  if (d.nx < 2 || d.ny < 2 || d.nz < 2) {
    return fail(MGB_ERR_UNSUPPORTED, "every axis needs at least 2 cells (reduced-dimension runs are refused)");
  }
  const int n[3] = {d.nx, d.ny, d.nz};
  for (int q = 0; q < 3; ++q) {
    if (d.E[q] == nullptr || d.D[q] == nullptr || d.B[q] == nullptr || d.inv_eps[q] == nullptr) {
      return fail(MGB_ERR_ARGUMENT, "a primary field or inverse-epsilon pointer is null");
    }
  }
  std::string why;
  if (d.pml_active) {
    for (int l = 0; l < 2; ++l)
      for (int a = 0; a < 3; ++a)
        if (d.kms[l][a] == nullptr || d.sinv[l][a] == nullptr || d.kps[l][a] == nullptr)
          return fail(MGB_ERR_ARGUMENT, "a PML coefficient vector is null");
    const int uaxis[3] = {2, 0, 1};
    for (int q = 0; q < 3; ++q) {
      if (!aux_ok(d.H[q], q, n[q], &why, "H", q) || !aux_ok(d.fwH[q], q, n[q], &why, "fwH", q) ||
          !aux_ok(d.fwE[q], q, n[q], &why, "fwE", q) ||
          !aux_ok(d.fuB[q], uaxis[q], n[uaxis[q]], &why, "fuB", q) ||
          !aux_ok(d.fuD[q], uaxis[q], n[uaxis[q]], &why, "fuD", q)) {
        return fail(MGB_ERR_ARGUMENT, why);
      }
    }
  }
  if (d.npoles < 0 || d.npoles > MGB_MAX_POLES) {
    return fail(MGB_ERR_UNSUPPORTED, "at most " + std::to_string(MGB_MAX_POLES) + " susceptibility poles are stepped");
  }
  if (d.npoles > 0) {
    for (int a = 0; a < 3; ++a) {
      if (d.pbox[2 * a] < 0 || d.pbox[2 * a] >= d.pbox[2 * a + 1] || d.pbox[2 * a + 1] > n[a]) {
        return fail(MGB_ERR_ARGUMENT, "polarization box is not inside the grid");
      }
    }
    for (int m = 0; m < d.npoles; ++m)
      for (int q = 0; q < 3; ++q)
        if (d.poles[m].sigma[q] != nullptr && (d.poles[m].p[q][0] == nullptr || d.poles[m].p[q][1] == nullptr))
          return fail(MGB_ERR_ARGUMENT, "a driven polarization component has no P buffers");
  }
  if (d.nsrc < 0 || (d.nsrc > 0 && (d.src_cell == nullptr || d.src_comp == nullptr))) {
    return fail(MGB_ERR_ARGUMENT, "source point tables are missing");
  }
  if (d.nmonitors < 0 || d.nmonitors > MGB_MAX_MONITORS) {
    return fail(MGB_ERR_UNSUPPORTED, "at most " + std::to_string(MGB_MAX_MONITORS) + " monitors per simulation");
  }
  for (int m = 0; m < d.nmonitors; ++m) {
    const mgb_monitor& mon = d.monitors[m];
    for (int a = 0; a < 3; ++a) {
      if (mon.region[2 * a] < 0 || mon.region[2 * a] >= mon.region[2 * a + 1] || mon.region[2 * a + 1] > n[a]) {
        return fail(MGB_ERR_ARGUMENT, "monitor " + std::to_string(m) + " region is not inside the grid");
      }
    }
    if (mon.ncomp < 1 || mon.ncomp > MGB_MAX_MONITOR_COMPONENTS || mon.nfreq < 1 ||
        mon.decimation < 1 || mon.omega == nullptr || mon.acc == nullptr) {
      return fail(MGB_ERR_ARGUMENT, "monitor " + std::to_string(m) + " is incomplete");
    }
    for (int q = 0; q < mon.ncomp; ++q) {
      if (mon.comp[q] < 0 || mon.comp[q] > 5) return fail(MGB_ERR_ARGUMENT, "monitor component out of range");
    }
    if ((size_t)mon.nfreq * 2 * sizeof(float2) > 48 * 1024) {
      return fail(MGB_ERR_UNSUPPORTED, "a monitor holds at most 3072 frequencies");
    }
  }
  mgb_sim* sim = new (std::nothrow) mgb_sim();
  if (sim == nullptr) return fail(MGB_ERR_ARGUMENT, "host allocation of the plan failed");
  sim->desc = d;
  StepParams& p = sim->step;
  p.nx = d.nx; p.ny = d.ny; p.nz = d.nz;
  for (int a = 0; a < 3; ++a) p.met[a] = d.metallic[a] ? 1 : 0;
  p.dtdx = d.dtdx;
  for (int l = 0; l < 2; ++l)
    for (int a = 0; a < 3; ++a) {
      p.kms[l][a] = d.kms[l][a];
      p.sinv[l][a] = d.sinv[l][a];
      p.kps[l][a] = d.kps[l][a];
    }
  for (int q = 0; q < 3; ++q) {
    p.E[q] = d.E[q]; p.D[q] = d.D[q]; p.B[q] = d.B[q]; p.inv_eps[q] = d.inv_eps[q];
    p.H[q] = d.H[q]; p.fwH[q] = d.fwH[q]; p.fwE[q] = d.fwE[q]; p.fuB[q] = d.fuB[q]; p.fuD[q] = d.fuD[q];
  }
  p.npoles = d.npoles;
  for (int a = 0; a < 6; ++a) { p.pbox[a] = d.pbox[a]; p.src_box[a] = d.src_box[a]; }
  for (int m = 0; m < d.npoles; ++m) p.poles[m] = d.poles[m];
  p.nsrc = d.nsrc;
  p.src_cell = d.src_cell;
  p.src_comp = d.src_comp;
  p.src_words = nullptr;
  p.status = d.status;
  *out = sim;
  return MGB_OK;
}

int mgb_set_launch_shape(mgb_sim* sim, int block_z, int block_y, int xchunk) {
  if (sim == nullptr) return fail(MGB_ERR_ARGUMENT, "null plan");
  if (block_z < 1 || block_y < 1 || block_z * block_y > 256 || xchunk < 1) {
    return fail(MGB_ERR_ARGUMENT, "launch shape needs block_z*block_y <= 256 and x_chunk >= 1");
  }
  sim->block_z = block_z;
  sim->block_y = block_y;
  sim->xchunk = xchunk;
  return MGB_OK;
}

int mgb_set_source_words(mgb_sim* sim, const double* words, int64_t first_step, int64_t steps) {
  if (sim == nullptr) return fail(MGB_ERR_ARGUMENT, "null plan");
  if (steps < 0 || (steps > 0 && words == nullptr)) return fail(MGB_ERR_ARGUMENT, "bad source word table");
  sim->words = words;
  sim->words_first = first_step;
  sim->words_steps = steps;
  return MGB_OK;
}

}  // extern "C"

namespace {

// Launches of one step, split by part so mgb_step and mgb_launch share them.
int launch_part(mgb_sim* sim, long long n, int part, cudaStream_t s) {
  StepParams& p = sim->step;
  const bool pml = sim->desc.pml_active != 0;
  if (part == 0 || part == 1) {
    if (p.nsrc > 0) p.src_words = sim->words + (n - sim->words_first) * p.nsrc;
    const dim3 block(sim->block_z, sim->block_y, 1);
    const dim3 grid((p.nz + block.x - 1) / block.x, (p.ny + block.y - 1) / block.y,
                    (p.nx + sim->xchunk - 1) / sim->xchunk);
    if (part == 0) {
      if (pml) h_half<true><<<grid, block, 0, s>>>(p, n == 0, sim->xchunk);
      else h_half<false><<<grid, block, 0, s>>>(p, n == 0, sim->xchunk);
    } else {
      if (pml) e_half<true><<<grid, block, 0, s>>>(p, (int)(n & 1), sim->xchunk);
      else e_half<false><<<grid, block, 0, s>>>(p, (int)(n & 1), sim->xchunk);
    }
    return MGB_OK;
  }
  const long long post = n + 1;
  for (int m = 0; m < sim->desc.nmonitors; ++m) {
    const mgb_monitor& mon = sim->desc.monitors[m];
    if (post % mon.decimation != 0) continue;
    DftParams q;
    q.nx = p.nx; q.ny = p.ny; q.nz = p.nz;
    for (int a = 0; a < 3; ++a) q.met[a] = p.met[a];
    q.pml = pml;
    for (int c = 0; c < 3; ++c) { q.E[c] = p.E[c]; q.B[c] = p.B[c]; q.H[c] = p.H[c]; }
    q.mon = mon;
    const long long cells = (long long)(mon.region[1] - mon.region[0]) *
                            (mon.region[3] - mon.region[2]) * (mon.region[5] - mon.region[4]);
    const unsigned blocks = (unsigned)((cells + 255) / 256);
    const size_t smem = (size_t)mon.nfreq * 2 * sizeof(float2);
    if (pml) dft_accumulate<true><<<blocks, 256, smem, s>>>(q, post);
    else dft_accumulate<false><<<blocks, 256, smem, s>>>(q, post);
  }
  return MGB_OK;
}

int check_words(mgb_sim* sim, long long first, long long count) {
  if (sim->step.nsrc > 0 &&
      (first < sim->words_first || first + count > sim->words_first + sim->words_steps)) {
    return fail(MGB_ERR_RANGE, "source words cover steps [" + std::to_string(sim->words_first) +
                                   ", " + std::to_string(sim->words_first + sim->words_steps) +
                                   ") but steps [" + std::to_string(first) + ", " +
                                   std::to_string(first + count) + ") were asked for");
  }
  return MGB_OK;
}

}  // namespace

extern "C" {

int mgb_step(mgb_sim* sim, int64_t first_step, int32_t nsteps, void* stream) {
  if (sim == nullptr) return fail(MGB_ERR_ARGUMENT, "null plan");
  if (nsteps < 0 || first_step < 0) return fail(MGB_ERR_ARGUMENT, "negative step range");
  if (nsteps == 0) return MGB_OK;
  const int rc = check_words(sim, first_step, nsteps);
  if (rc != MGB_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  for (int32_t t = 0; t < nsteps; ++t) {
    const long long n = first_step + t;
    for (int part = 0; part < 3; ++part) launch_part(sim, n, part, s);
    if (t == 0) {
      const int err = launch_error("step launch");
      if (err != MGB_OK) return err;
    }
  }
  return launch_error("step launch");
}

int mgb_launch(mgb_sim* sim, int64_t step, int32_t part, void* stream) {
  if (sim == nullptr) return fail(MGB_ERR_ARGUMENT, "null plan");
  if (step < 0 || part < 0 || part > 2) return fail(MGB_ERR_ARGUMENT, "bad step or part");
  if (part < 2) {
    const int rc = check_words(sim, step, 1);
    if (rc != MGB_OK) return rc;
  }
  launch_part(sim, step, part, static_cast<cudaStream_t>(stream));
  return launch_error("launch");
}

int mgb_flux_spectrum(mgb_sim* sim, int32_t monitor, const float* weights, double* out,
                      void* stream) {
  if (sim == nullptr || weights == nullptr || out == nullptr) return fail(MGB_ERR_ARGUMENT, "null argument");
  if (monitor < 0 || monitor >= sim->desc.nmonitors) return fail(MGB_ERR_ARGUMENT, "no such monitor");
  const mgb_monitor& m = sim->desc.monitors[monitor];
  if (m.ncomp != 4 || m.comp[0] > 2 || m.comp[1] > 2 || m.comp[2] < 3 || m.comp[3] < 3) {
    return fail(MGB_ERR_ARGUMENT, "monitor is not a flux plane (Ea, Eb, Ha, Hb)");
  }
  flux_reduce<<<m.nfreq, 256, 0, static_cast<cudaStream_t>(stream)>>>(m, weights, out);
  return launch_error("flux reduction launch");
}

void mgb_destroy(mgb_sim* sim) { delete sim; }

}  // extern "C"
