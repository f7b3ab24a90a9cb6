// meepgb.cu — GB300 (sm_103a) FDTD stepping kernels and the C ABI of libmeepgb.so.
//
// One step is two fused kernels:
//   H half: MEEP's step_B (curl E with the split-field UPML), zero_metal_B and
//           update_H (own-axis constitutive accumulation);
//   E half: step_D, the electric source deposit in double, zero_metal_D, update_E
//           (chi1inv of D minus every polarization, own-axis accumulation) and update_P
//           (Lorentz/Drude ADE), all on the registers of one cell;
// followed on decimated steps by dft_accumulate for every monitor.
//
// Arithmetic follows the reference array path operation for operation (meep_gpu/
// stepping.py: _curl_from_operands :2265, _apply_pml_update :2629,
// _apply_dsig_only_update :2662, _apply_constitutive_pml :2991, separate_h_from_b
// :2789, _mask_non_owned_cells :2589, _zero_metal :3135; dispersion.py
// PolarizationState.update :689; sources.py _deposit :1357). The file is compiled
// with -fmad=false so no multiply-add is contracted: every float32 word equals the
// reference's separately rounded operations.
//
// Storage: E, D and H are full volumes. MEEP's H is B's own word outside each H
// component's own-axis PML membership, so B is stored only on that membership (a
// compact slab) and H carries it everywhere else. Every PML auxiliary is a compact slab
// over its membership runs.
//
// Two kernel families share that layout:
//   tile kernels (h_tile, e_tile): a CTA owns a 64 (z) x 8 (y) tile and marches over a
//     chunk of x planes. One thread issues TMA bulk-tensor loads (cp.async.bulk.tensor)
//     of each plane's tiles (the stencil operand with its one-cell halo, the cell's own
//     fields) into a ring of shared-memory stages guarded by mbarriers, several planes
//     ahead of the 512 threads (one per tile cell) computing from shared memory; the x
//     neighbour is the previous (or next) stage of the ring. Waits are bounded: a wait that outlives its
//     limit sets status bit 2 and the CTA stops stepping.
//   generic kernels (h_generic, e_generic): one thread per (y, z) column marching over
//     x with plain loads, for grids whose z extent is not a multiple of 4 (TMA needs
//     16-byte row strides).

#include "meepgb.h"
#include "dft_tc.cuh"
#include "reduced.cuh"
#include "wave.cuh"

#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <utility>
#include <mutex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

thread_local std::string g_error;

int fail(int code, const std::string& message) {
  g_error = message;
  return code;
}

// Test hook (mgb_set_test_wait_limit): the limit, in nanoseconds, of the first bounded
// wait of the next launches of the tile kernels (index 0: their first shared-memory stage)
// and of the tensor-core contraction (index 1: its first tile's MMAs); negative keeps the
// normal limit. Every later wait of those kernels, the drains included, keeps its normal
// bound.
std::atomic<long long> g_test_wait_limit[2] = {{-1}, {-1}};

long long test_wait_limit(int which) { return g_test_wait_limit[which].load(std::memory_order_relaxed); }

constexpr int kTileZ = 64;          // cells per tile along z (innermost)
constexpr int kTileY = 8;           // cells per tile along y
constexpr int kHaloZ = kTileZ + 4;  // z extent of a halo box (16-byte multiple)
constexpr int kHaloY = kTileY + 1;
constexpr int kThreads = 512;         // one thread per tile cell
constexpr int kBoxHalo = 2560;      // bytes of one halo box buffer (68 x 9 floats, 128-aligned)
constexpr int kBoxOwn = kTileZ * kTileY * 4;  // 2048 bytes

}  // namespace

#include "step_device.cuh"

using namespace mgbstep;

namespace {


template <bool PML, bool MSRC>
__global__ void __launch_bounds__(256, 4) h_generic_pf(const __grid_constant__ StepParams p,
                                                       int first_step, int xchunk) {
  step_entry();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (k >= p.nz || j >= p.ny) return;
  const int i0 = (blockIdx.z + p.xbase) * xchunk, i1 = min(i0 + xchunk, p.nx);
  // a run with magnetic sources: the CTAs that hold source points deposit them
  if (MSRC && cta_msrc(p, i0, i1, blockIdx.y * blockDim.y, blockDim.y, blockIdx.x * blockDim.x, blockDim.x)) {
    h_march_pf<PML, -1, true>(p, j, k, i0, i1, first_step);
    return;
  }
  if (!PML) {
    h_march_pf<false>(p, j, k, i0, i1, first_step);
    return;
  }
#define MGB_MARCH(AXV, PMLV) h_march_pf<PMLV, AXV>(p, j, k, i0, i1, first_step)
  MGB_AXES_SWITCH(cta_axes(p, i0, i1, blockIdx.y * blockDim.y, blockDim.y, blockIdx.x * blockDim.x, blockDim.x),
                  MGB_MARCH)
#undef MGB_MARCH
}

template <bool PML>
__global__ void __launch_bounds__(256, 4) e_generic_pf(const __grid_constant__ StepParams p, int parity,
                                                       int xchunk) {
  step_entry();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (k >= p.nz || j >= p.ny) return;
  const int i0 = (blockIdx.z + p.xbase) * xchunk, i1 = min(i0 + xchunk, p.nx);
  if (!PML) {
    e_march_pf<false>(p, j, k, i0, i1, parity, p.src_words);
    return;
  }
#define MGB_MARCH(AXV, PMLV) e_march_pf<PMLV, AXV>(p, j, k, i0, i1, parity, p.src_words)
  MGB_AXES_SWITCH(cta_axes(p, i0, i1, blockIdx.y * blockDim.y, blockDim.y, blockIdx.x * blockDim.x, blockDim.x),
                  MGB_MARCH)
#undef MGB_MARCH
}

// Generic kernels: plain loads, one thread per (y, z) column marching over an x chunk.
template <bool PML, bool MSRC>
__global__ void __launch_bounds__(256, 5) h_generic(const __grid_constant__ StepParams p,
                                                    int first_step, int xchunk) {
  step_entry();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (k >= p.nz || j >= p.ny) return;
  const int i0 = (blockIdx.z + p.xbase) * xchunk, i1 = min(i0 + xchunk, p.nx);
  // a Bloch-phased run: the CTAs at index 0 of a phased axis read the other part there
  if (cta_bloch(p, i0, blockIdx.y * blockDim.y, blockIdx.x * blockDim.x)) {
    h_march<PML, false, -1, true, true>(p, j, k, i0, i1, first_step);
    return;
  }
  // a run with magnetic sources: the CTAs that hold source points deposit them
  if (MSRC && cta_msrc(p, i0, i1, blockIdx.y * blockDim.y, blockDim.y, blockIdx.x * blockDim.x, blockDim.x)) {
    h_march<PML, false, -1, true>(p, j, k, i0, i1, first_step);
    return;
  }
  if (!PML) {
    h_march<false>(p, j, k, i0, i1, first_step);
    return;
  }
  // one march compiled for exactly the axes whose memberships the CTA reaches
#define MGB_MARCH(AXV, PMLV) h_march<PMLV, false, AXV>(p, j, k, i0, i1, first_step)
  MGB_AXES_SWITCH(cta_axes(p, i0, i1, blockIdx.y * blockDim.y, blockDim.y, blockIdx.x * blockDim.x, blockDim.x),
                  MGB_MARCH)
#undef MGB_MARCH
}

template <bool PML>
__global__ void __launch_bounds__(256, 5) e_generic(const __grid_constant__ StepParams p, int parity,
                                                    int xchunk) {
  step_entry();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (k >= p.nz || j >= p.ny) return;
  const int i0 = (blockIdx.z + p.xbase) * xchunk, i1 = min(i0 + xchunk, p.nx);
  // a Bloch-phased run: the CTAs at index 0 of a phased axis read the other part there
  if (cta_bloch(p, i0, blockIdx.y * blockDim.y, blockIdx.x * blockDim.x)) {
    e_march<PML, false, -1, true>(p, j, k, i0, i1, parity, p.src_words);
    return;
  }
  if (!PML) {
    e_march<false>(p, j, k, i0, i1, parity, p.src_words);
    return;
  }
  // one march compiled for exactly the axes whose memberships the CTA reaches
#define MGB_MARCH(AXV, PMLV) e_march<PMLV, false, AXV>(p, j, k, i0, i1, parity, p.src_words)
  MGB_AXES_SWITCH(cta_axes(p, i0, i1, blockIdx.y * blockDim.y, blockDim.y, blockIdx.x * blockDim.x, blockDim.x),
                  MGB_MARCH)
#undef MGB_MARCH
}

// Generic kernels of a lossy run (a D or B conductivity): the same column march with
// the conductive curl forms; the conductivity volumes and tables come as a second
// parameter block so the lossless kernels' parameters stay as they are.
template <bool PML, bool MSRC>
__global__ void __launch_bounds__(256, 4) h_generic_cond(const __grid_constant__ StepParams p,
                                                      const __grid_constant__ mgb_conductivity cp,
                                                      int first_step, int xchunk) {
  step_entry();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (k >= p.nz || j >= p.ny) return;
  const int i0 = (blockIdx.z + p.xbase) * xchunk, i1 = min(i0 + xchunk, p.nx);
  // a Bloch-phased run: the CTAs at index 0 of a phased axis read the other part there
  if (cta_bloch(p, i0, blockIdx.y * blockDim.y, blockIdx.x * blockDim.x)) {
    h_march<PML, true, -1, true, true>(p, j, k, i0, i1, first_step, &cp);
    return;
  }
  // a run with magnetic sources: the CTAs that hold source points deposit them
  if (MSRC && cta_msrc(p, i0, i1, blockIdx.y * blockDim.y, blockDim.y, blockIdx.x * blockDim.x, blockDim.x)) {
    h_march<PML, true, -1, true>(p, j, k, i0, i1, first_step, &cp);
    return;
  }
  if (!PML) {
    h_march<false, true>(p, j, k, i0, i1, first_step, &cp);
    return;
  }
#define MGB_MARCH(AXV, PMLV) h_march<PMLV, true, AXV>(p, j, k, i0, i1, first_step, &cp)
  MGB_AXES_SWITCH(cta_axes(p, i0, i1, blockIdx.y * blockDim.y, blockDim.y, blockIdx.x * blockDim.x, blockDim.x),
                  MGB_MARCH)
#undef MGB_MARCH
}

template <bool PML>
__global__ void __launch_bounds__(256, 4) e_generic_cond(const __grid_constant__ StepParams p,
                                                      const __grid_constant__ mgb_conductivity cp,
                                                      int parity, int xchunk) {
  step_entry();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (k >= p.nz || j >= p.ny) return;
  const int i0 = (blockIdx.z + p.xbase) * xchunk, i1 = min(i0 + xchunk, p.nx);
  // a Bloch-phased run: the CTAs at index 0 of a phased axis read the other part there
  if (cta_bloch(p, i0, blockIdx.y * blockDim.y, blockIdx.x * blockDim.x)) {
    e_march<PML, true, -1, true>(p, j, k, i0, i1, parity, p.src_words, &cp);
    return;
  }
  if (!PML) {
    e_march<false, true>(p, j, k, i0, i1, parity, p.src_words, &cp);
    return;
  }
#define MGB_MARCH(AXV, PMLV) e_march<PMLV, true, AXV>(p, j, k, i0, i1, parity, p.src_words, &cp)
  MGB_AXES_SWITCH(cta_axes(p, i0, i1, blockIdx.y * blockDim.y, blockDim.y, blockIdx.x * blockDim.x, blockDim.x),
                  MGB_MARCH)
#undef MGB_MARCH
}

// ------------------------------------------------------------------------------------
// TMA + mbarrier primitives (inline PTX).
__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

constexpr unsigned long long kStageWaitNs = 2000000000ull;  // ~2 s of wall time

// Wait for phase `parity` of a stage barrier, for at most limit_ns of wall time; a limit
// of 0 gives up without looking (the test hook that makes a wait run out).
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity,
                                          unsigned long long limit_ns = kStageWaitNs) {
  if (limit_ns == 0) return false;
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long start = global_ns();
  for (;;) {
    for (int spin = 0; spin < 256; ++spin)
      if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - start > limit_ns) return false;
  }
}

__device__ __forceinline__ unsigned long long first_stage_limit(const TileMaps& maps) {
  return maps.first_wait_ns >= 0 ? (unsigned long long)maps.first_wait_ns : kStageWaitNs;
}

__device__ __forceinline__ void tma_load(void* dst, const CUtensorMap* map,
                                         unsigned long long* bar, int z, int y, int x) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(smem_addr(bar)), "r"(z), "r"(y), "r"(x)
      : "memory");
}

// After an aborted wait: thread 0 lets this CTA's copies still in flight land (each
// wait bounded) before the CTA exits and its shared memory is reused. `from` is the
// oldest chain not yet known to have landed in every thread; waiting again on a chain
// that has landed returns at once (its stage's phase has completed).
__device__ __noinline__ void drain_copies(unsigned long long* full, int S, int from, int issued,
                                          int tid) {
  if (tid != 0) return;
  for (int c = from; c < issued; ++c) mbar_wait(&full[c % S], (unsigned)((c / S) & 1));
}

// ------------------------------------------------------------------------------------
// Tile kernels. Per plane: every thread waits (bounded) for the plane's stage, computes
// its cell from shared memory, and the CTA meets at one barrier, after which thread 0
// refills the stage the CTA has finished with. A wait that times out makes its thread
// skip the cell and raise the shared abort flag, which every thread reads after the
// barrier, so the whole CTA leaves together.
//
// H half. Ring stage of chain index c (plane i0 + c): the E box (68 x 9, z from k0 and
// y from j0, so the +1 halo of the forward differences) and, for planes below i1, the
// cell's own H box. Plane i1 (the chunk's x neighbour above) carries E only; past the
// high x face it is the zero fill of a metallic wall or plane 0 of a periodic axis.
// Past the high y or z face of a periodic axis the halo is row or column 0, which the
// box does not hold: those cells read it from global memory.
template <bool PML>
__global__ void __launch_bounds__(kThreads, 2) h_tile(const __grid_constant__ StepParams p,
                                                     const __grid_constant__ TileMaps maps,
                                                     int first_step, int xchunk) {
  step_entry();
  extern __shared__ __align__(128) unsigned char smem[];
  const int S = maps.stages;
  const int stage_bytes = 3 * kBoxHalo + 3 * kBoxOwn;
  unsigned long long* full = reinterpret_cast<unsigned long long*>(smem + S * stage_bytes);
  __shared__ int abort_flag;
  const int tid = threadIdx.x;
  const int k0 = blockIdx.x * kTileZ, j0 = blockIdx.y * kTileY;
  const int i0 = blockIdx.z * xchunk;
  const int i1 = min(i0 + xchunk, p.nx);
  const int nchain = i1 - i0 + 1;  // planes i0 .. i1
  auto issue = [&](int chain) {
    const int st = chain % S;
    unsigned char* base = smem + st * stage_bytes;
    const int plane = i0 + chain;
    const bool own = plane < i1;
    const int xplane = (plane >= p.nx && !p.met[0]) ? plane - p.nx : plane;
    mbar_expect_tx(&full[st], 3 * (kHaloZ * kHaloY * 4) + (own ? 3 * kBoxOwn : 0));
    for (int q = 0; q < 3; ++q) tma_load(base + q * kBoxHalo, &maps.E[q], &full[st], k0, j0, xplane);
    if (own)
      for (int q = 0; q < 3; ++q)
        tma_load(base + 3 * kBoxHalo + q * kBoxOwn, &maps.Hown[q], &full[st], k0, j0, plane);
  };
  int issued = 0;  // chains issued so far (meaningful in thread 0)
  if (tid == 0) {
    abort_flag = 0;
    for (int st = 0; st < S; ++st) mbar_init(&full[st], 1);
    mbar_fence_init();
    for (int c = 0; c < S && c < nchain; ++c) issue(c);
    issued = S < nchain ? S : nchain;
  }
  __syncthreads();
  const int tz = tid & (kTileZ - 1), ty = tid / kTileZ;
  const int j = j0 + ty, k = k0 + tz;
  const bool live = j < p.ny && k < p.nz;
  HColumn hcol = {};
  int col_axes = 0;  // bit 1: the warp touches the y memberships, bit 2: the z ones
  if (PML) {
    if (live) hcol = h_column(p, j, k);
    col_axes = (__any_sync(0xffffffffu, live && (hcol.f2 || hcol.b1)) ? 2 : 0) |
               (__any_sync(0xffffffffu, live && (hcol.f0 || hcol.b2)) ? 4 : 0);
  }
  const bool wrap_y = live && !p.met[1] && j + 1 == p.ny;
  const bool wrap_z = live && !p.met[2] && k + 1 == p.nz;
  const int sx = p.ny * p.nz;
  const int col = j * p.nz + k;
  const int e = ty * kHaloZ + tz;  // this cell in an E box
  const int o = ty * kTileZ + tz;  // this cell in an own box
  const float dtdx = p.dtdx;
  bool ok = mbar_wait(&full[0], 0, first_stage_limit(maps));
  for (int i = i0; i < i1; ++i) {
    const int chain = i - i0;
    ok = ok && mbar_wait(&full[(chain + 1) % S], (unsigned)(((chain + 1) / S) & 1));
    if (!ok) {
      abort_flag = 1;
    } else if (live) {
      const float* st0 = reinterpret_cast<const float*>(smem + (chain % S) * stage_bytes);
      const float* st1 = reinterpret_cast<const float*>(smem + ((chain + 1) % S) * stage_bytes);
      const float* Ex0 = st0;
      const float* Ey0 = st0 + kBoxHalo / 4;
      const float* Ez0 = st0 + 2 * kBoxHalo / 4;
      const float* Hown = st0 + 3 * kBoxHalo / 4;
      const int c = i * sx + col;
      const float ex = Ex0[e], ey = Ey0[e], ez = Ez0[e];
      float ez_yp = Ez0[e + kHaloZ], ex_yp = Ex0[e + kHaloZ];
      float ey_zp = Ey0[e + 1], ex_zp = Ex0[e + 1];
      if (wrap_y) { ez_yp = p.E[2][c - (p.ny - 1) * p.nz]; ex_yp = p.E[0][c - (p.ny - 1) * p.nz]; }
      if (wrap_z) { ey_zp = p.E[1][c - (p.nz - 1)]; ex_zp = p.E[0][c - (p.nz - 1)]; }
      const float cx = dtdx * (((ez_yp - ez) + ey) - ey_zp);
      const float cy = dtdx * (((ex_zp - ex) + ez) - (st1 + 2 * kBoxHalo / 4)[e]);
      const float cz = dtdx * ((((st1 + kBoxHalo / 4)[e] - ey) + ex) - ex_yp);
      const float h_old[3] = {Hown[o], Hown[kBoxOwn / 4 + o], Hown[2 * kBoxOwn / 4 + o]};
      float h_new[3];
      HPlane pl = {};
      int axes = 0;
      if (PML) {
        pl = h_plane(p, i);
        axes = col_axes | ((pl.f1 || pl.b0) ? 1 : 0);
        if (h_needs_plane(axes)) h_plane_coefficients(p, i, pl);
      }
      HAux ax = {};
      if (PML && axes != 0) h_aux_load(p, hcol, pl, c, ax);
      h_cell<PML, false, -1, true>(p, hcol, pl, axes, first_step, i, j, k, c, cx, cy, cz, h_old, ax, h_new);
      p.H[0][c] = h_new[0];
      p.H[1][c] = h_new[1];
      p.H[2][c] = h_new[2];
    }
    __syncthreads();  // the stage of plane i is read by everyone
    if (abort_flag) {
      // chains chain .. issued - 1 may still be in flight (chain itself when the wait
      // that failed was the first one)
      if (p.status != nullptr && tid == 0) atomicOr(p.status, 2);
      drain_copies(full, S, chain, issued, tid);
      return;
    }
    if (tid == 0 && chain + S < nchain) {
      fence_proxy_async_smem();
      issue(chain + S);
      issued = chain + S + 1;
    }
  }
}

// E half. Ring stage of chain index c (plane i0 - 1 + c): the H box (68 x 9, z from
// k0 - 4 and y from j0 - 1, so the -1 halo of the backward differences) and, for planes
// at or above i0, the cell's own D and inverse-epsilon boxes. Plane i0 - 1 (the chunk's
// x neighbour below) carries H only; below the low x face it is the zero fill of a
// metallic wall or plane nx - 1 of a periodic axis. Below the low y or z face of a
// periodic axis the halo is row ny - 1 or column nz - 1: those cells read it from
// global memory.
template <bool PML>
__global__ void __launch_bounds__(kThreads, 2) e_tile(const __grid_constant__ StepParams p,
                                                     const __grid_constant__ TileMaps maps,
                                                     int parity, int xchunk) {
  step_entry();
  extern __shared__ __align__(128) unsigned char smem[];
  const int S = maps.stages;
  const int stage_bytes = 3 * kBoxHalo + (3 + maps.ninv) * kBoxOwn;
  unsigned long long* full = reinterpret_cast<unsigned long long*>(smem + S * stage_bytes);
  __shared__ int abort_flag;
  const int tid = threadIdx.x;
  const int k0 = blockIdx.x * kTileZ, j0 = blockIdx.y * kTileY;
  const int i0 = blockIdx.z * xchunk;
  const int i1 = min(i0 + xchunk, p.nx);
  const int nchain = i1 - i0 + 1;  // planes i0-1 .. i1-1
  auto issue = [&](int chain) {
    const int st = chain % S;
    unsigned char* base = smem + st * stage_bytes;
    const int plane = i0 - 1 + chain;
    const bool own = plane >= i0;
    const int xplane = (plane < 0 && !p.met[0]) ? plane + p.nx : plane;
    mbar_expect_tx(&full[st], 3 * (kHaloZ * kHaloY * 4) + (own ? (3 + maps.ninv) * kBoxOwn : 0));
    for (int q = 0; q < 3; ++q)
      tma_load(base + q * kBoxHalo, &maps.Hhalo[q], &full[st], k0 - 4, j0 - 1, xplane);
    if (own) {
      for (int q = 0; q < 3; ++q)
        tma_load(base + 3 * kBoxHalo + q * kBoxOwn, &maps.D[q], &full[st], k0, j0, plane);
      for (int q = 0; q < maps.ninv; ++q)
        tma_load(base + 3 * kBoxHalo + (3 + q) * kBoxOwn, &maps.inv[q], &full[st], k0, j0, plane);
    }
  };
  int issued = 0;  // chains issued so far (meaningful in thread 0)
  if (tid == 0) {
    abort_flag = 0;
    for (int st = 0; st < S; ++st) mbar_init(&full[st], 1);
    mbar_fence_init();
    for (int c = 0; c < S && c < nchain; ++c) issue(c);
    issued = S < nchain ? S : nchain;
  }
  __syncthreads();
  const int tz = tid & (kTileZ - 1), ty = tid / kTileZ;
  const int j = j0 + ty, k = k0 + tz;
  const bool live = j < p.ny && k < p.nz;
  EColumn ecol = {};
  int col_axes = 0;  // bit 1: the warp touches the y memberships, bit 2: the z ones
  if (PML) {
    if (live) ecol = e_column(p, j, k);
    col_axes = (__any_sync(0xffffffffu, live && (ecol.f2 || ecol.w1)) ? 2 : 0) |
               (__any_sync(0xffffffffu, live && (ecol.f0 || ecol.w2)) ? 4 : 0);
  }
  const bool wrap_y = live && !p.met[1] && j == 0;
  const bool wrap_z = live && !p.met[2] && k == 0;
  const int sx = p.ny * p.nz;
  const int col = j * p.nz + k;
  const int h = (ty + 1) * kHaloZ + tz + 4;  // this cell in an H box
  const int o = ty * kTileZ + tz;            // this cell in an own box
  const int inv0 = 3 + maps.inv_of[0], inv1 = 3 + maps.inv_of[1], inv2 = 3 + maps.inv_of[2];
  const float dtdx = p.dtdx;
  bool ok = mbar_wait(&full[0], 0, first_stage_limit(maps));
  for (int i = i0; i < i1; ++i) {
    const int chain = i - i0 + 1;
    ok = ok && mbar_wait(&full[chain % S], (unsigned)((chain / S) & 1));
    if (!ok) {
      abort_flag = 1;
    } else if (live) {
      const float* st1 = reinterpret_cast<const float*>(smem + (chain % S) * stage_bytes);
      const float* st0 = reinterpret_cast<const float*>(smem + ((chain - 1) % S) * stage_bytes);
      const float* Hx = st1;
      const float* Hy = st1 + kBoxHalo / 4;
      const float* Hz = st1 + 2 * kBoxHalo / 4;
      const float* own = st1 + 3 * kBoxHalo / 4;
      const int c = i * sx + col;
      const float hx = Hx[h], hy = Hy[h], hz = Hz[h];
      float hz_ym = Hz[h - kHaloZ], hx_ym = Hx[h - kHaloZ];
      float hy_zm = Hy[h - 1], hx_zm = Hx[h - 1];
      if (wrap_y) { hz_ym = p.H[2][c + (p.ny - 1) * p.nz]; hx_ym = p.H[0][c + (p.ny - 1) * p.nz]; }
      if (wrap_z) { hy_zm = p.H[1][c + (p.nz - 1)]; hx_zm = p.H[0][c + (p.nz - 1)]; }
      const float cx = dtdx * (((hz_ym - hz) + hy) - hy_zm);
      const float cy = dtdx * (((hx_zm - hx) + hz) - (st0 + 2 * kBoxHalo / 4)[h]);
      const float cz = dtdx * ((((st0 + kBoxHalo / 4)[h] - hy) + hx) - hx_ym);
      float d[3] = {own[o], own[kBoxOwn / 4 + o], own[2 * kBoxOwn / 4 + o]};
      const float inv[3] = {own[inv0 * (kBoxOwn / 4) + o], own[inv1 * (kBoxOwn / 4) + o],
                            own[inv2 * (kBoxOwn / 4) + o]};
      EPlane pl = {};
      int axes = 0;
      if (PML) {
        pl = e_plane(p, i);
        axes = col_axes | ((pl.f1 || pl.w0) ? 1 : 0);
        if (axes & 1) e_plane_coefficients(p, i, pl);
      }
      EAux ax = {};
      if (PML && axes != 0) e_aux_load(p, ecol, pl, c, ax);
      e_cell<PML>(p, ecol, pl, axes, parity, i, j, k, c, cx, cy, cz, d, inv, p.src_words, ax);
    }
    __syncthreads();  // the stage of plane i - 1 is read by everyone
    if (abort_flag) {
      // chains chain - 1 .. issued - 1 may still be in flight (chain - 1 when the wait
      // that failed was the first one)
      if (p.status != nullptr && tid == 0) atomicOr(p.status, 2);
      drain_copies(full, S, chain - 1, issued, tid);
      return;
    }
    if (tid == 0 && chain - 1 + S < nchain) {
      fence_proxy_async_smem();
      issue(chain - 1 + S);
      issued = chain - 1 + S + 1;
    }
  }
}

// ------------------------------------------------------------------------------------
// Warp-specialized tile kernel (E half): the tile kernels' staging, with one producer
// warp that keeps the ring of plane stages full (it waits on each stage's "empty"
// barrier, then issues the plane's TMA loads against its "full" barrier) and 16
// consumer warps that each wait only for the stage they need and release the stage of
// the plane before once they are done with it. No CTA-wide barrier in the plane loop:
// each consumer warp runs ahead as far as the data allows. Waits are bounded (2 s); a
// timeout raises the shared abort flag and status bit 2, consumers leave, and the
// producer waits (bounded) for its copies still in flight before it leaves.
constexpr int kWsThreads = kThreads + 32;

__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

template <bool PML>
__global__ void __launch_bounds__(kWsThreads, 2) e_ws(const __grid_constant__ StepParams p,
                                                     const __grid_constant__ TileMaps maps,
                                                     int parity, int xchunk) {
  step_entry();
  extern __shared__ __align__(128) unsigned char smem[];
  const int S = maps.stages;
  const int stage_bytes = 3 * kBoxHalo + (3 + maps.ninv) * kBoxOwn;
  unsigned long long* full = reinterpret_cast<unsigned long long*>(smem + S * stage_bytes);
  unsigned long long* empty = full + S;
  __shared__ int abort_flag;
  const int tid = threadIdx.x;
  const int k0 = blockIdx.x * kTileZ, j0 = blockIdx.y * kTileY;
  const int i0 = blockIdx.z * xchunk;
  const int i1 = min(i0 + xchunk, p.nx);
  const int nchain = i1 - i0 + 1;  // planes i0-1 .. i1-1
  if (tid == 0) {
    abort_flag = 0;
    for (int st = 0; st < S; ++st) {
      mbar_init(&full[st], 1);
      mbar_init(&empty[st], kThreads / 32);
    }
    mbar_fence_init();
  }
  __syncthreads();
  if (tid >= kThreads) {
    // producer warp: one lane issues
    if (tid == kThreads) {
      int issued = 0;
      for (int c = 0; c < nchain; ++c) {
        const int st = c % S;
        if (c >= S && !mbar_wait(&empty[st], (unsigned)(((c / S) - 1) & 1))) {
          atomicExch(&abort_flag, 1);
          break;
        }
        if (*reinterpret_cast<volatile int*>(&abort_flag)) break;
        fence_proxy_async_smem();
        unsigned char* base = smem + st * stage_bytes;
        const int plane = i0 - 1 + c;
        const bool own = plane >= i0;
        const int xplane = (plane < 0 && !p.met[0]) ? plane + p.nx : plane;
        mbar_expect_tx(&full[st], 3 * (kHaloZ * kHaloY * 4) + (own ? (3 + maps.ninv) * kBoxOwn : 0));
        for (int q = 0; q < 3; ++q)
          tma_load(base + q * kBoxHalo, &maps.Hhalo[q], &full[st], k0 - 4, j0 - 1, xplane);
        if (own) {
          for (int q = 0; q < 3; ++q)
            tma_load(base + 3 * kBoxHalo + q * kBoxOwn, &maps.D[q], &full[st], k0, j0, plane);
          for (int q = 0; q < maps.ninv; ++q)
            tma_load(base + 3 * kBoxHalo + (3 + q) * kBoxOwn, &maps.inv[q], &full[st], k0, j0, plane);
        }
        issued = c + 1;
      }
      // no copy may land after the CTA has left: wait (bounded) for the last ones
      for (int c = issued > S ? issued - S : 0; c < issued; ++c)
        mbar_wait(&full[c % S], (unsigned)((c / S) & 1));
    }
    return;
  }
  const int tz = tid & (kTileZ - 1), ty = tid / kTileZ;
  const int j = j0 + ty, k = k0 + tz;
  const bool live = j < p.ny && k < p.nz;
  EColumn ecol = {};
  int col_axes = 0;  // bit 1: the warp touches the y memberships, bit 2: the z ones
  if (PML) {
    if (live) ecol = e_column(p, j, k);
    col_axes = (__any_sync(0xffffffffu, live && (ecol.f2 || ecol.w1)) ? 2 : 0) |
               (__any_sync(0xffffffffu, live && (ecol.f0 || ecol.w2)) ? 4 : 0);
  }
  const bool wrap_y = live && !p.met[1] && j == 0;
  const bool wrap_z = live && !p.met[2] && k == 0;
  const int sx = p.ny * p.nz;
  const int col = j * p.nz + k;
  const int h = (ty + 1) * kHaloZ + tz + 4;  // this cell in an H box
  const int o = ty * kTileZ + tz;            // this cell in an own box
  const int inv0 = 3 + maps.inv_of[0], inv1 = 3 + maps.inv_of[1], inv2 = 3 + maps.inv_of[2];
  const float dtdx = p.dtdx;
  bool ok = __all_sync(0xffffffffu, mbar_wait(&full[0], 0));
  for (int i = i0; i < i1 && ok; ++i) {
    const int chain = i - i0 + 1;
    ok = __all_sync(0xffffffffu, mbar_wait(&full[chain % S], (unsigned)((chain / S) & 1)));
    if (!ok) break;
    if (live) {
      const float* st1 = reinterpret_cast<const float*>(smem + (chain % S) * stage_bytes);
      const float* st0 = reinterpret_cast<const float*>(smem + ((chain - 1) % S) * stage_bytes);
      const float* Hx = st1;
      const float* Hy = st1 + kBoxHalo / 4;
      const float* Hz = st1 + 2 * kBoxHalo / 4;
      const float* own = st1 + 3 * kBoxHalo / 4;
      const int c = i * sx + col;
      EPlane pl = {};
      int axes = 0;
      if (PML) {
        pl = e_plane(p, i);
        axes = col_axes | ((pl.f1 || pl.w0) ? 1 : 0);
        if (axes & 1) e_plane_coefficients(p, i, pl);
      }
      EAux ax = {};
      if (PML && axes != 0) e_aux_load(p, ecol, pl, c, ax);
      const float hx = Hx[h], hy = Hy[h], hz = Hz[h];
      float hz_ym = Hz[h - kHaloZ], hx_ym = Hx[h - kHaloZ];
      float hy_zm = Hy[h - 1], hx_zm = Hx[h - 1];
      if (wrap_y) { hz_ym = p.H[2][c + (p.ny - 1) * p.nz]; hx_ym = p.H[0][c + (p.ny - 1) * p.nz]; }
      if (wrap_z) { hy_zm = p.H[1][c + (p.nz - 1)]; hx_zm = p.H[0][c + (p.nz - 1)]; }
      const float cx = dtdx * (((hz_ym - hz) + hy) - hy_zm);
      const float cy = dtdx * (((hx_zm - hx) + hz) - (st0 + 2 * kBoxHalo / 4)[h]);
      const float cz = dtdx * ((((st0 + kBoxHalo / 4)[h] - hy) + hx) - hx_ym);
      float d[3] = {own[o], own[kBoxOwn / 4 + o], own[2 * kBoxOwn / 4 + o]};
      const float inv[3] = {own[inv0 * (kBoxOwn / 4) + o], own[inv1 * (kBoxOwn / 4) + o],
                            own[inv2 * (kBoxOwn / 4) + o]};
      e_cell<PML>(p, ecol, pl, axes, parity, i, j, k, c, cx, cy, cz, d, inv, p.src_words, ax);
    }
    // the stage of plane i - 1 is no longer read by this warp
    __syncwarp();
    if ((tid & 31) == 0) mbar_arrive(&empty[(chain - 1) % S]);
    if (*reinterpret_cast<volatile int*>(&abort_flag)) ok = false;
  }
  if (!ok) {
    atomicExch(&abort_flag, 1);
    if (p.status != nullptr && (tid & 31) == 0) atomicOr(p.status, 2);
  }
}

// ------------------------------------------------------------------------------------
// DFT accumulation on one monitor: cell-centred samples times float64-formed phases.
__device__ __forceinline__ float field_at(const DftParams& p, int comp, int i, int j, int k) {
  // A monitor's ladder may reach past a periodic face (MEEP's lattice-image gather): the
  // ladder point r samples stored cell r mod n, one lattice vector (or more) away from
  // it; past a metallic face the wall holds zero.
  const int n[3] = {p.nx, p.ny, p.nz};
  if (p.fold) {
    // A folded axis (MEEP's sn loop, reference dft.py:1004): site r of a component with
    // Yee shift s sits at doubled -2 + 2r + s. Outside the unfolded cell's owned window
    // it reads zero past a metallic face, or its image one lattice vector over past a
    // periodic one; below the plane it is the image at -d with the component's parity;
    // past the stored rows it is zero (a metallic far wall) or the image about the second
    // mirror at doubled full (a periodic face), with the parity again.
    int at[3] = {i, j, k};
    bool flip = false;
    const int q = comp % 3;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (!((p.fold >> a) & 1)) {
        if (at[a] < 0 || at[a] >= n[a]) {
          if (p.met[a]) return 0.f;
          at[a] %= n[a];
          if (at[a] < 0) at[a] += n[a];
        }
        continue;
      }
      const int s = (comp < 3) == (a == q) ? 1 : 0;
      const bool periodic = (p.far >> a) & 1;
      const bool odd = (p.neg[comp] >> a) & 1;
      const int low = -(p.full[a] - p.full[a] % 2), lattice = 2 * p.full[a];
      int d = -2 + 2 * at[a] + s;
      if (d < low + 2 - s || d > low + lattice - s) {
        if (!periodic) return 0.f;
        d += d < low + 2 - s ? lattice : -lattice;
        if (d < low + 2 - s || d > low + lattice - s) return 0.f;
      }
      if (d < -s) {
        d = -d;
        if (odd) flip = !flip;
      }
      int row = (d + 2 - s) >> 1;
      if (row >= n[a]) {
        if (!periodic) return 0.f;
        d = lattice - d;
        if (odd) flip = !flip;
        row = (d + 2 - s) >> 1;
        if (d + 2 - s < 0 || row >= n[a]) return 0.f;
      }
      at[a] = row;
    }
    const long long c = ((long long)at[0] * p.ny + at[1]) * p.nz + at[2];
    const float own = comp < 3 ? p.E[comp][c] : p.H[comp - 3][c];
    return flip ? -own : own;
  }
  const int raw[3] = {i, j, k};
  int at[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    int r = raw[a];
    if (r < 0 || r >= n[a]) {
      if (p.met[a]) return 0.f;
      r %= n[a];
      if (r < 0) r += n[a];
    }
    at[a] = r;
  }
  const long long c = ((long long)at[0] * p.ny + at[1]) * p.nz + at[2];
  const float own = comp < 3 ? p.E[comp][c] : p.H[comp - 3][c];
  if (!p.bloch) return own;
  // On a Bloch-phased axis the ladder point is eikna^count times the stored word, count
  // the lattice vectors between them: floor((r - low) / n), low = 1 for a component with
  // Yee shift 0 there (its cell 0 stores MEEP's owned top point) and 0 otherwise.
  const int q = comp % 3;
  float fr = 1.f, fi = 0.f;
  bool any = false;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (!((p.bloch >> a) & 1)) continue;
    const int low = (comp < 3 ? (a != q) : (a == q)) ? 1 : 0;
    const int shifted = raw[a] - low;
    int count = shifted >= 0 ? shifted / n[a] : -((-shifted + n[a] - 1) / n[a]);
    const float br = p.bre[a], bi = count < 0 ? -p.bim[a] : p.bim[a];
    for (count = count < 0 ? -count : count; count > 0; --count) {
      const float nr = fr * br - fi * bi, ni = fr * bi + fi * br;
      fr = nr;
      fi = ni;
      any = true;
    }
  }
  if (!any) return own;
  const float other = comp < 3 ? p.pE[comp][c] : p.pH[comp - 3][c];
  return p.part ? (fr * own) + (fi * other) : (fr * own) - (fi * other);
}

// Yee-to-centre average along every axis where the component's shift is 0, x then y
// then z, each 0.5*(f[i] + f[i+1]) in float32 (reference dft.py:352).
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
      const float f0 = field_at(p, comp, i, j + a, k + b);
      v[b][a] = ax ? 0.5f * (f0 + field_at(p, comp, i + 1, j + a, k + b)) : f0;
    }
  }
  float r0 = ay ? 0.5f * (v[0][0] + v[0][1]) : v[0][0];
  if (!az) return r0;
  float r1 = ay ? 0.5f * (v[1][0] + v[1][1]) : v[1][0];
  return 0.5f * (r0 + r1);
}

// The float64-formed phases of one accumulation into shared memory: [0, nf) for E at
// t = step*dt, [nf, 2nf) for H at t - dt/2 (the caller synchronises).
__device__ __forceinline__ void dft_phases(const mgb_monitor& m, long long step, float2* phase) {
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
}

// Accumulate one region cell of one monitor.
__device__ __forceinline__ void dft_cell(const DftParams& p, const float2* phase, long long cell) {
  const mgb_monitor& m = p.mon;
  const int nf = m.nfreq;
  const int rx = m.region[1] - m.region[0], ry = m.region[3] - m.region[2],
            rz = m.region[5] - m.region[4];
  const long long cells = (long long)rx * ry * rz;
  if (cell >= cells) return;
  const int rk = (int)(cell % rz);
  const int rj = (int)((cell / rz) % ry);
  const int ri = (int)(cell / ((long long)ry * rz));
  const int i = m.region[0] + ri, j = m.region[2] + rj, k = m.region[4] + rk;
  for (int q = 0; q < m.ncomp; ++q) {
    const int comp = m.comp[q];
    const float s = centred(p, comp, i, j, k);
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

__global__ void __launch_bounds__(256) dft_accumulate(const __grid_constant__ DftParams p,
                                                      long long step) {
  extern __shared__ float2 phase[];  // [0, nf): E phases, [nf, 2nf): H phases
  dft_phases(p.mon, step, phase);
  __syncthreads();
  dft_cell(p, phase, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// Buffered (tensor-core) accumulation: write one decimated step's cell-centred samples
// of every component into row `row` of the monitor's sample buffer [depth][ncomp * cells].
__global__ void __launch_bounds__(256) dft_sample(const __grid_constant__ DftParams p, float* row) {
  const mgb_monitor& m = p.mon;
  const int rx = m.region[1] - m.region[0], ry = m.region[3] - m.region[2],
            rz = m.region[5] - m.region[4];
  const long long cells = (long long)rx * ry * rz;
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= cells) return;
  const int rk = (int)(cell % rz);
  const int rj = (int)((cell / rz) % ry);
  const int ri = (int)(cell / ((long long)ry * rz));
  const int i = m.region[0] + ri, j = m.region[2] + rj, k = m.region[4] + rk;
  for (int q = 0; q < m.ncomp; ++q) row[(long long)q * cells + cell] = centred(p, m.comp[q], i, j, k);
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

// ------------------------------------------------------------------------------------
// Batched stepping of many independent simulations (serving). A slot table holds every
// admitted simulation's step parameters; a work list cuts every active slot's grid into
// (slot, z tile, y tile, x chunk) items of the batch's launch shape, one CTA each. A CTA
// copies its slot's parameters into shared memory and runs the generic column march on
// them, so a slot computes the words of the same simulation stepped alone.
//
// Step counters live on the host: every running slot advances exactly one step per batch
// step, so before each call of G steps the host uploads each slot's step at the start
// (n0), and launch t of the G computes n = n0 + t. A slot whose n has reached its end is
// skipped by every kernel, so one captured graph of G steps is replayed while slots
// finish at different steps, and slots coming and going change only the tables, the lists
// and the launches' grid sizes. Three launches per step: H half, E half, monitors.
//
// (Measured on GB300 against two other layouts of the same march: a resident grid
// looping over the list needs 78-80 registers a thread and loses occupancy; the slot
// table in constant memory, indexed by the CTA's slot, misses the constant cache. Both
// stepped a 128^3 slot 10-15 % slower than this one.)
constexpr int kSlotMonitors = 2;
constexpr int kBatchMaxFreq = 512;
constexpr int kDftItemCells = 256;

struct SlotState {
  long long end;        // the slot has run all its steps when n reaches end
  const double* words;  // deposit words [end][nsrc] from step 0
  int active;
  int nmon;
};

struct BatchTables {
  StepParams* params;  // [max_slots]
  SlotState* state;    // [max_slots]
  long long* n0;       // [max_slots] step of each slot at the first launch of a batch step call
  DftParams* dft;      // [max_slots * kSlotMonitors]
  int4* work;          // step items (slot, z tile, y tile, x chunk)
  int4* dft_work;      // monitor items (slot * kSlotMonitors + monitor, cell block)
  int* counts;         // [0] step items, [1] monitor items
  int max_slots;
  int xchunk;          // x cells per step item; the block is (z, y) cells
};

template <typename T>
__device__ __forceinline__ void copy_to_shared(T* dst, const T* src) {
  static_assert(sizeof(T) % 4 == 0, "copied as 32-bit words");
  const int* from = reinterpret_cast<const int*>(src);
  int* to = reinterpret_cast<int*>(dst);
  const int n = (int)(sizeof(T) / 4);
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  for (int i = tid; i < n; i += blockDim.x * blockDim.y) to[i] = from[i];
}

// GEN false: the prefetching marches (family 2, 64 registers); true: the generic marches
// with each item's x chunk prefetched into L2 (family 4, 48 registers). `t` is the
// launch's step within the batch step call.
// The phased march of a batched Bloch slot's CTA (one half of step n).
template <int PART>
__device__ __noinline__ void batched_bloch_march(const StepParams& sp, int j, int k, int i0, int i1, long long n,
                                                 const double* slot_words) {
  if (PART == 0) {
    if (sp.pml) h_march<true, false, -1, true, true>(sp, j, k, i0, i1, n == 0);
    else h_march<false, false, -1, true, true>(sp, j, k, i0, i1, n == 0);
  } else {
    const double* words = slot_words + n * sp.nsrc;
    if (sp.pml) e_march<true, false, -1, true>(sp, j, k, i0, i1, (int)(n & 1), words);
    else e_march<false, false, -1, true>(sp, j, k, i0, i1, (int)(n & 1), words);
  }
}

// The H march of a batched slot's CTA that holds magnetic source points (step n's row of
// the slot's words is in the shared parameters).
__device__ __noinline__ void batched_msrc_march(const StepParams& sp, int j, int k, int i0, int i1, long long n) {
  if (sp.pml) h_march<true, false, -1, true>(sp, j, k, i0, i1, n == 0);
  else h_march<false, false, -1, true>(sp, j, k, i0, i1, n == 0);
}

template <int PART, bool GEN>
__global__ void __launch_bounds__(256, GEN ? 5 : 4) step_batched(const __grid_constant__ BatchTables tb, int t) {
  __shared__ StepParams sp;
  if ((int)blockIdx.x >= tb.counts[0]) return;
  const int4 w = tb.work[blockIdx.x];
  // The parameter copy and the slot's state are fetched together (one round trip).
  copy_to_shared(&sp, &tb.params[w.x]);
  const SlotState st = tb.state[w.x];
  const long long n = tb.n0[w.x] + t;
  if (!st.active || n >= st.end) return;  // uniform over the CTA
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    sp.l2pf = GEN ? 1 : 0;
    sp.src_words = st.words != nullptr ? st.words + n * sp.nsrc : nullptr;  // step n's row
  }
  __syncthreads();
  const int k = w.y * (int)blockDim.x + (int)threadIdx.x;
  const int j = w.z * (int)blockDim.y + (int)threadIdx.y;
  if (k >= sp.nz || j >= sp.ny) return;
  const int i0 = w.w * tb.xchunk;
  const int i1 = min(i0 + tb.xchunk, sp.nx);
  const int axes = sp.pml ? cta_axes(sp, i0, i1, w.z * (int)blockDim.y, (int)blockDim.y,
                                      w.y * (int)blockDim.x, (int)blockDim.x) : 0;
  // a Bloch-phased slot (one part of a complex run, its other part in another slot of the
  // same batch step): the CTAs at index 0 of a phased axis read the other part there
  // (out of line, so the other marches keep their register allocation)
  if (cta_bloch(sp, i0, w.z * (int)blockDim.y, w.y * (int)blockDim.x)) {
    batched_bloch_march<PART>(sp, j, k, i0, i1, n, st.words);
    return;
  }
  // a slot with magnetic sources: the CTAs that hold its magnetic points deposit them
  if (PART == 0 && cta_msrc(sp, i0, i1, w.z * (int)blockDim.y, (int)blockDim.y, w.y * (int)blockDim.x,
                            (int)blockDim.x)) {
    batched_msrc_march(sp, j, k, i0, i1, n);
    return;
  }
  if (PART == 0) {
    const int first = n == 0;
    if (GEN) {
#define MGB_MARCH(AXV, PMLV) h_march<PMLV, false, AXV>(sp, j, k, i0, i1, first)
      MGB_AXES_SWITCH(axes, MGB_MARCH)
#undef MGB_MARCH
    } else {
#define MGB_MARCH(AXV, PMLV) h_march_pf<PMLV, AXV>(sp, j, k, i0, i1, first)
      MGB_AXES_SWITCH(axes, MGB_MARCH)
#undef MGB_MARCH
    }
  } else {
    const double* words = st.words + n * sp.nsrc;
    const int parity = (int)(n & 1);
    if (GEN) {
#define MGB_MARCH(AXV, PMLV) e_march<PMLV, false, AXV>(sp, j, k, i0, i1, parity, words)
      MGB_AXES_SWITCH(axes, MGB_MARCH)
#undef MGB_MARCH
    } else {
#define MGB_MARCH(AXV, PMLV) e_march_pf<PMLV, AXV>(sp, j, k, i0, i1, parity, words)
      MGB_AXES_SWITCH(axes, MGB_MARCH)
#undef MGB_MARCH
    }
  }
}

__global__ void __launch_bounds__(kDftItemCells) dft_batched(const __grid_constant__ BatchTables tb, int t) {
  __shared__ float2 phase[2 * kBatchMaxFreq];
  __shared__ DftParams dp;
  if ((int)blockIdx.x >= tb.counts[1]) return;
  const int4 w = tb.dft_work[blockIdx.x];
  const int slot = w.x / kSlotMonitors;
  copy_to_shared(&dp, &tb.dft[w.x]);
  const SlotState st = tb.state[slot];
  const long long n = tb.n0[slot] + t;
  if (!st.active || n >= st.end) return;
  __syncthreads();
  // Monitors are due after step n when (n + 1) is a multiple of their decimation.
  const long long post = n + 1;
  if (post % dp.mon.decimation != 0) return;
  dft_phases(dp.mon, post, phase);
  __syncthreads();
  dft_cell(dp, phase, (long long)w.y * kDftItemCells + threadIdx.x);
}

// ------------------------------------------------------------------------------------
// Adjoint (reverse-time) step: the transpose of one forward step, for gradients of a
// flux objective with respect to the inverse permittivity. The adjoint state has the
// forward state's layout (a second plan whose field and auxiliary pointers are the
// adjoint arrays, with the forward's coefficient tables, memberships and inverse
// permittivity). The forward step is linear in its state; each half is a local update
// of every cell from its old words and a curl of the other family, so its transpose is
// the transposed local update, which yields the adjoint of the curl input ("mu"), and
// the transposed curl, a gather of mu from the neighbours:
//   forward H half: curl = dtdx * C(E) (forward differences), then the B/H update;
//   forward E half: curl = dtdx * C'(H) (backward differences), then the D/E update.
// Reversing forward step n: kernel adj_e (E half) first adds dtdx * C^T(mu_B) of step
// n + 1 into the adjoint of E, then runs the transposed E update, stores mu_D and adds
// the gradient dJ/d(inv_eps) += (adjoint of w) * D' over the design box (w = inv * D'
// is where the inverse permittivity enters); kernel adj_h then adds dtdx * C'^T(mu_D)
// into the adjoint of H and runs the transposed B/H update, storing mu_B. Every
// coefficient outside its membership is exactly 1, so the general forms serve every
// cell. No poles (the caller refuses them). Derivations per operation are in comments.
struct AdjParams {
  float* mu_b[3];      // adjoint of the H half's curl input, per B component
  float* mu_d[3];      // adjoint of the E half's curl input, per D component
  int box[6];          // gradient box, half-open
  const float* d_after;  // [3][box cells]: forward D after the step being reversed
  float* grad_inv;       // [box cells]
  int first_step;        // the step being reversed is step 0 (separate_h_from_b)
};

__device__ __forceinline__ float coef(const float* table, bool pml, int at) {
  return pml ? __ldg(table + at) : 1.f;
}

__device__ __forceinline__ constexpr bool axis_on(int ax, int a) { return ax >= 0 && ((ax >> a) & 1) != 0; }

// The reverse marches below are compiled per CTA for the axes whose memberships the CTA
// reaches (AX, as the forward kernels are; -1 with PML false: none): along any other axis
// every membership is empty and every coefficient exactly 1 for the CTA's cells, so those
// loads and tests drop out and the words are those of the general form. The x
// neighbours of mu carry from plane to plane in registers, and the chunk's planes are
// requested into L2 before the march.

// One thread's column (j, k) of the reverse E half over planes [i0, i1): gather mu_B,
// transposed D/E update, mu_D, gradient.
template <bool PML, int AX>
__device__ __forceinline__ void adj_e_march(const StepParams& p, const AdjParams& a, int j, int k, int i0, int i1) {
  const int sx = p.ny * p.nz, sy = p.nz;
  const float dtdx = p.dtdx;
  // "c - y": the cell whose forward (+y) neighbour is this one: none on a metallic
  // axis at 0, the last row on a periodic one.
  const int jm = j > 0 ? j - 1 : (p.met[1] ? -1 : p.ny - 1);
  const int km = k > 0 ? k - 1 : (p.met[2] ? -1 : p.nz - 1);
  const int box_ny = a.box[3] - a.box[2], box_nz = a.box[5] - a.box[4];
  const bool jk_in_box = j >= a.box[2] && j < a.box[3] && k >= a.box[4] && k < a.box[5];
  const long long box_cells = (long long)(a.box[1] - a.box[0]) * box_ny * box_nz;
  const int col = j * sy + k;
  {
    const float* vols[12] = {p.E[0], p.E[1], p.E[2], p.D[0], p.D[1], p.D[2],
                             a.mu_b[0], a.mu_b[1], a.mu_b[2], p.inv_eps[0], p.inv_eps[1], p.inv_eps[2]};
    prefetch_planes(vols, p.inv_eps[1] == p.inv_eps[0] ? 10 : 12, i0 * sx + col, sx, i1 - i0);
  }
  // mu_B of y and z components one plane below (x neighbours), carried
  float mb1_xm = 0.f, mb2_xm = 0.f;
  {
    const int im = i0 > 0 ? i0 - 1 : (p.met[0] ? -1 : p.nx - 1);
    if (im >= 0) {
      mb1_xm = a.mu_b[1][im * sx + col];
      mb2_xm = a.mu_b[2][im * sx + col];
    }
  }
  for (int i = i0; i < i1; ++i) {
    const int c = i * sx + col;
    const int cym = jm >= 0 ? i * sx + jm * sy + k : -1;
    const int czm = km >= 0 ? i * sx + j * sy + km : -1;
    const int coord[3] = {i, j, k};
    const bool in_box = jk_in_box && i >= a.box[0] && i < a.box[1];
    const long long bcell =
        in_box ? ((long long)(i - a.box[0]) * box_ny + (j - a.box[2])) * box_nz + (k - a.box[4]) : 0;
    // Every word the cell reads, before any store: the stores of one component could
    // alias the next one's loads for all the compiler knows, so loads placed between
    // them would each wait a round trip; gathered here they are one.
    bool own[3], fm[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      own[q] = PML && axis_on(AX, q) && in_runs(p.fwE[q], coord[q]);
      fm[q] = PML && axis_on(AX, (q + 2) % 3) && in_runs(p.fuD[q], coord[(q + 2) % 3]);
    }
    auto mb = [&](int q, int at) { return at >= 0 ? a.mu_b[q][at] : 0.f; };
    const float mb0 = a.mu_b[0][c], mb1 = a.mu_b[1][c], mb2 = a.mu_b[2][c];
    const float mb1_zm = mb(1, czm), mb2_ym = mb(2, cym), mb0_zm = mb(0, czm), mb0_ym = mb(0, cym);
    float e_old[3], d_old[3], inv[3], fw_old[3], fu_old[3], d_after[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      e_old[q] = p.E[q][c];
      d_old[q] = p.D[q][c];
      inv[q] = p.inv_eps[q][c];
      fw_old[q] = own[q] ? p.fwE[q].data[c] : 0.f;
      fu_old[q] = fm[q] ? p.fuD[q].data[c] : 0.f;
      d_after[q] = in_box ? a.d_after[(long long)q * box_cells + bcell] : 0.f;
    }
    const float grad_old = in_box ? a.grad_inv[bcell] : 0.f;
    // Transpose of the H half's curls (forward differences):
    //   cx = dtdx*((Ez[+y] - Ez) + Ey - Ey[+z]), cy = dtdx*((Ex[+z] - Ex) + Ez - Ez[+x]),
    //   cz = dtdx*((Ey[+x] - Ey) + Ex - Ex[+y]).
    float le[3];
    le[0] = e_old[0] + dtdx * ((mb1_zm - mb1) + (mb2 - mb2_ym));
    le[1] = e_old[1] + dtdx * ((mb0 - mb0_zm) + (mb2_xm - mb2));
    le[2] = e_old[2] + dtdx * ((mb0_ym - mb0) + (mb1 - mb1_xm));
    mb1_xm = mb1;
    mb2_xm = mb2;
    const bool wx = p.met[0] && i == 0, wy = p.met[1] && j == 0, wz = p.met[2] && k == 0;
    float grad = 0.f;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const int a1 = (q + 1) % 3, a2 = (q + 2) % 3;
      const bool masked = q == 0 ? (wy || wz) : q == 1 ? (wx || wz) : (wx || wy);
      const bool c1 = PML && axis_on(AX, a1), c2 = PML && axis_on(AX, a2);
      const float k1 = coef(p.kms[kInteger][a1], c1, coord[a1]);
      const float s1 = coef(p.sinv[kInteger][a1], c1, coord[a1]);
      const float k2 = coef(p.kms[kInteger][a2], c2, coord[a2]);
      const float s2 = coef(p.sinv[kInteger][a2], c2, coord[a2]);
      // E' = E + (kps*w - kms*fw), fw' = w on the own membership; E' = w elsewhere.
      float lw = le[q], le_in = 0.f;
      if (own[q]) {
        const float kps = __ldg(p.kps[kHalf][q] + coord[q]);
        const float kms = __ldg(p.kms[kHalf][q] + coord[q]);
        lw = kps * le[q] + fw_old[q];
        le_in = le[q];
        p.fwE[q].data[c] = -kms * le[q];
      }
      if (in_box) grad += lw * d_after[q];
      // w = inv * d'; D' = d'; d' is forced to 0 on the masked wall cells.
      const float ld = masked ? 0.f : d_old[q] + inv[q] * lw;
      // d' from the curl: split-field recurrence on the dsigu membership, else
      // d' = (k1*d - curl)*s1. fu' is stored even on masked cells (curl 0 there).
      float ld_in, mu;
      if (fm[q]) {
        const float ln = s2 * ld + fu_old[q];
        ld_in = k2 * s2 * ld;
        p.fuD[q].data[c] = -s2 * ld + k1 * s1 * ln;
        mu = -s1 * ln;
      } else {
        ld_in = k1 * s1 * ld;
        mu = -s1 * ld;
      }
      p.D[q][c] = ld_in;
      p.E[q][c] = le_in;
      a.mu_d[q][c] = masked ? 0.f : mu;
    }
    if (in_box) a.grad_inv[bcell] = grad_old + grad;
  }
}

// One thread's column (j, k) of the reverse H half over planes [i0, i1): gather mu_D,
// transposed B/H update, mu_B.
template <bool PML, int AX>
__device__ __forceinline__ void adj_h_march(const StepParams& p, const AdjParams& a, int j, int k, int i0, int i1) {
  const int sx = p.ny * p.nz, sy = p.nz;
  const float dtdx = p.dtdx;
  // "c + y": the cell whose backward (-y) neighbour is this one: none on a metallic axis
  // at the top, row 0 on a periodic one.
  const int jp = j + 1 < p.ny ? j + 1 : (p.met[1] ? -1 : 0);
  const int kp = k + 1 < p.nz ? k + 1 : (p.met[2] ? -1 : 0);
  const int col = j * sy + k;
  {
    const float* vols[6] = {p.H[0], p.H[1], p.H[2], a.mu_d[0], a.mu_d[1], a.mu_d[2]};
    prefetch_planes(vols, 6, i0 * sx + col, sx, i1 - i0);
  }
  // mu_D of y and z components at this plane, carried from the plane below's x neighbour
  float md1 = a.mu_d[1][i0 * sx + col], md2 = a.mu_d[2][i0 * sx + col];
  for (int i = i0; i < i1; ++i) {
    const int ip = i + 1 < p.nx ? i + 1 : (p.met[0] ? -1 : 0);
    const int c = i * sx + col;
    const int cyp = jp >= 0 ? i * sx + jp * sy + k : -1;
    const int czp = kp >= 0 ? i * sx + j * sy + kp : -1;
    const int cxp = ip >= 0 ? ip * sx + col : -1;
    const int coord[3] = {i, j, k};
    // every word the cell reads, before any store (one round trip, as in the E half)
    bool own[3], fm[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      own[q] = PML && axis_on(AX, q) && in_runs(p.B[q], coord[q]);
      fm[q] = PML && axis_on(AX, (q + 2) % 3) && in_runs(p.fuB[q], coord[(q + 2) % 3]);
    }
    auto md = [&](int q, int at) { return at >= 0 ? a.mu_d[q][at] : 0.f; };
    const float md0 = a.mu_d[0][c];
    const float md1_xp = md(1, cxp), md2_xp = md(2, cxp);
    const float md1_zp = md(1, czp), md2_yp = md(2, cyp), md0_zp = md(0, czp), md0_yp = md(0, cyp);
    float h_old[3], fw_old[3], b_old[3], fu_old[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      h_old[q] = p.H[q][c];
      fw_old[q] = own[q] ? p.fwH[q].data[c] : 0.f;
      b_old[q] = own[q] ? p.B[q].data[c] : 0.f;
      fu_old[q] = fm[q] ? p.fuB[q].data[c] : 0.f;
    }
    // Transpose of the E half's curls (backward differences):
    //   cx = dtdx*((Hz[-y] - Hz) + Hy - Hy[-z]), cy = dtdx*((Hx[-z] - Hx) + Hz - Hz[-x]),
    //   cz = dtdx*((Hy[-x] - Hy) + Hx - Hx[-y]).
    float lh[3];
    lh[0] = h_old[0] + dtdx * ((md1_zp - md1) + (md2 - md2_yp));
    lh[1] = h_old[1] + dtdx * ((md0 - md0_zp) + (md2_xp - md2));
    lh[2] = h_old[2] + dtdx * ((md0_yp - md0) + (md1 - md1_xp));
    md1 = md1_xp;
    md2 = md2_xp;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const int a1 = (q + 1) % 3, a2 = (q + 2) % 3;
      // zero_metal_B: the curl and the new word of B_q are 0 at index 0 of a metallic
      // own axis (never an own-axis membership cell).
      const bool wall = p.met[q] && coord[q] == 0;
      const bool c1 = PML && axis_on(AX, a1), c2 = PML && axis_on(AX, a2);
      const float k1 = coef(p.kms[kHalf][a1], c1, coord[a1]);
      const float s1 = coef(p.sinv[kHalf][a1], c1, coord[a1]);
      const float k2 = coef(p.kms[kHalf][a2], c2, coord[a2]);
      const float s2 = coef(p.sinv[kHalf][a2], c2, coord[a2]);
      // H' = H + (kps*b' - kms*fw) (step 0: b' + (kps*b' - kms*b')), fw' = b', B' = b' on
      // the own membership; elsewhere H' = b' and H's storage is B's word.
      float lb;
      float lh_in = 0.f, lw_in = 0.f;
      if (own[q]) {
        const float kps = __ldg(p.kps[kInteger][q] + coord[q]);
        const float kms = __ldg(p.kms[kInteger][q] + coord[q]);
        const float extra = fw_old[q] + b_old[q];
        if (a.first_step) {
          lb = ((1.f + kps) - kms) * lh[q] + extra;
        } else {
          lb = kps * lh[q] + extra;
          lh_in = lh[q];
          lw_in = -kms * lh[q];
        }
      } else {
        lb = wall ? 0.f : lh[q];
      }
      float lb_in, mu;
      if (fm[q]) {
        const float ln = s2 * lb + fu_old[q];
        lb_in = k2 * s2 * lb;
        p.fuB[q].data[c] = -s2 * lb + k1 * s1 * ln;
        mu = -s1 * ln;
      } else {
        lb_in = k1 * s1 * lb;
        mu = -s1 * lb;
      }
      if (own[q]) {
        p.B[q].data[c] = lb_in;
        p.H[q][c] = lh_in;
        p.fwH[q].data[c] = lw_in;
      } else {
        p.H[q][c] = lb_in;
      }
      a.mu_b[q][c] = wall ? 0.f : mu;
    }
  }
}

// Reverse of the E half, one CTA per (z, y) tile and x chunk.
template <bool PML>
__global__ void __launch_bounds__(256) adj_e(const __grid_constant__ StepParams p,
                                             const __grid_constant__ AdjParams a, int xchunk) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (k >= p.nz || j >= p.ny) return;
  const int i0 = blockIdx.z * xchunk, i1 = min(i0 + xchunk, p.nx);
  if (!PML) {
    adj_e_march<false, -1>(p, a, j, k, i0, i1);
    return;
  }
#define MGB_MARCH(AXV, PMLV) adj_e_march<PMLV, AXV>(p, a, j, k, i0, i1)
  MGB_AXES_SWITCH(cta_axes(p, i0, i1, blockIdx.y * blockDim.y, blockDim.y, blockIdx.x * blockDim.x, blockDim.x),
                  MGB_MARCH)
#undef MGB_MARCH
}

// Reverse of the H half.
template <bool PML>
__global__ void __launch_bounds__(256) adj_h(const __grid_constant__ StepParams p,
                                             const __grid_constant__ AdjParams a, int xchunk) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (k >= p.nz || j >= p.ny) return;
  const int i0 = blockIdx.z * xchunk, i1 = min(i0 + xchunk, p.nx);
  if (!PML) {
    adj_h_march<false, -1>(p, a, j, k, i0, i1);
    return;
  }
#define MGB_MARCH(AXV, PMLV) adj_h_march<PMLV, AXV>(p, a, j, k, i0, i1)
  MGB_AXES_SWITCH(cta_axes(p, i0, i1, blockIdx.y * blockDim.y, blockDim.y, blockIdx.x * blockDim.x, blockDim.x),
                  MGB_MARCH)
#undef MGB_MARCH
}

// Adjoint of one DFT sample taken after step post - 1: the sample's adjoint
// g_q(c) = sum_f (cos(w_f t) scale * coef[q][f][0][c] + sin(w_f t) scale * coef[q][f][1][c])
// (t at the component's time, coef in the accumulator layout) is spread back over the
// Yee words the centred sample averaged, with the same weights (atomic adds: samples of
// neighbouring cells share words).
__device__ __forceinline__ void scatter_centred(const DftParams& p, int comp, int i, int j, int k, float g) {
  const int q = comp % 3;
  const bool electric = comp < 3;
  const bool ax = electric ? (q != 0) : (q == 0);
  const bool ay = electric ? (q != 1) : (q == 1);
  const bool az = electric ? (q != 2) : (q == 2);
  const float w = (ax ? 0.5f : 1.f) * (ay ? 0.5f : 1.f) * (az ? 0.5f : 1.f);
  float* base = electric ? const_cast<float*>(p.E[q]) : const_cast<float*>(p.H[q]);
  for (int b = 0; b <= (az ? 1 : 0); ++b)
    for (int a = 0; a <= (ay ? 1 : 0); ++a)
      for (int d = 0; d <= (ax ? 1 : 0); ++d) {
        int ii = i + d, jj = j + a, kk = k + b;
        if (ii >= p.nx) { if (p.met[0]) continue; ii -= p.nx; }
        if (jj >= p.ny) { if (p.met[1]) continue; jj -= p.ny; }
        if (kk >= p.nz) { if (p.met[2]) continue; kk -= p.nz; }
        atomicAdd(base + ((long long)ii * p.ny + jj) * p.nz + kk, g * w);
      }
}

__global__ void __launch_bounds__(256) adj_inject(const __grid_constant__ DftParams p, long long post) {
  extern __shared__ float2 phase[];  // [0, nf): E phases, [nf, 2nf): H phases
  dft_phases(p.mon, post, phase);
  __syncthreads();
  const mgb_monitor& m = p.mon;
  const int nf = m.nfreq;
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
    const float2* ph = comp < 3 ? phase : phase + nf;
    const float* cf = m.acc + (long long)q * nf * 2 * cells + cell;
    float g = 0.f;
    for (int f = 0; f < nf; ++f) g += ph[f].x * cf[(long long)(2 * f) * cells] + ph[f].y * cf[(long long)(2 * f + 1) * cells];
    if (g != 0.f) scatter_centred(p, comp, i, j, k, g);
  }
}

// One accumulator component as interleaved complex64: planar rows [nf][2][cells] (re,
// im) of the real-part plan, and of the imaginary-part plan when `b` is not null.
__global__ void __launch_bounds__(256) interleave_accumulator(const float* __restrict__ a,
                                                              const float* __restrict__ b, long long nf,
                                                              long long cells, float2* __restrict__ dst) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf * cells) return;
  const long long f = t / cells, c = t - f * cells;
  const float* ra = a + f * 2 * cells;
  float re = ra[c], im = ra[cells + c];
  if (b != nullptr) {
    const float* rb = b + f * 2 * cells;
    re = re - rb[cells + c];
    im = im + rb[c];
  }
  dst[t] = make_float2(re, im);
}

// Copy [3][box] of one field family (0 E, 1 D, 2 H) into dst.
__global__ void __launch_bounds__(256) copy_box(const __grid_constant__ StepParams p, int family,
                                                BoxArgs b) {
  const long long cells = (long long)(b.box[1] - b.box[0]) * (b.box[3] - b.box[2]) * (b.box[5] - b.box[4]);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * cells) return;
  const int q = (int)(t / cells);
  const long long cell = t % cells;
  const int bz = b.box[5] - b.box[4], by = b.box[3] - b.box[2];
  const int k = b.box[4] + (int)(cell % bz);
  const int j = b.box[2] + (int)((cell / bz) % by);
  const int i = b.box[0] + (int)(cell / ((long long)by * bz));
  const float* src = family == 0 ? p.E[q] : family == 1 ? p.D[q] : p.H[q];
  b.dst[t] = src[((long long)i * p.ny + j) * p.nz + k];
}

// ------------------------------------------------------------------------------------
// Mirror folds (reference stepping.py:2004-2045 fill_symmetry_bc_B/D). Cell 0 of a
// component with Yee shift 0 on a folded axis is the plane's ghost: the step kernels
// treat it as a metallic wall sample (curl masked, as MEEP's owned-cell loop skips it),
// and after the half's sources it becomes the parity-signed word of stored row 2 (the
// product of the parities at a corner), then zero_metal of the other axes' walls, and
// its E (H) is stepped from that word with the ghost's own coefficients. The step
// kernels have by then overwritten the ghost's E, D and P (H and B) from the wall word,
// so each ghost's state from before the half is kept in `saved` (words [w * count + t]:
// E, its f_w formed from the old D and P, and P; H and B's old word as its f_w):
// the H fold kernel keeps the D ghosts' state for the E half that follows, the E fold
// kernel the B ghosts' state for the next step's H half.

__device__ __forceinline__ void cell_of(const StepParams& p, int c, int& i, int& j, int& k) {
  const int sx = p.ny * p.nz;
  i = c / sx;
  const int r = c - i * sx;
  j = r / p.nz;
  k = r - j * p.nz;
}

__device__ __forceinline__ int coord_along(int q, int i, int j, int k) { return q == 0 ? i : q == 1 ? j : k; }

__device__ __forceinline__ long long pole_index(const StepParams& p, int i, int j, int k, bool& in_box) {
  in_box = p.npoles > 0 && i >= p.pbox[0] && i < p.pbox[1] && j >= p.pbox[2] && j < p.pbox[3] &&
           k >= p.pbox[4] && k < p.pbox[5];
  if (!in_box) return 0;
  const int bny = p.pbox[3] - p.pbox[2], bnz = p.pbox[5] - p.pbox[4];
  return ((long long)(i - p.pbox[0]) * bny + (j - p.pbox[2])) * bnz + (k - p.pbox[4]);
}

// The B ghosts' H and f_w before the H half.
__device__ __forceinline__ void fold_keep_h(const StepParams& p, const FoldArgs& f, int t) {
  const int n = f.count[0], g = f.ghost[0][t], q = f.code[0][t] & 3;
  int i, j, k;
  cell_of(p, g, i, j, k);
  const bool sb = p.pml && in_runs(p.B[q], coord_along(q, i, j, k));
  f.saved[0][t] = p.H[q][g];
  f.saved[0][n + t] = sb ? p.B[q].data[g] : 0.f;  // f_w of H is B's word there
}

// The D ghosts' E, f_w and the polarization the E half overwrites, before the E half.
__device__ __forceinline__ void fold_keep_e(const StepParams& p, const FoldArgs& f, int t, int parity) {
  const int n = f.count[1], g = f.ghost[1][t], q = f.code[1][t] & 3;
  int i, j, k;
  cell_of(p, g, i, j, k);
  const bool sw = p.pml && in_runs(p.fwE[q], coord_along(q, i, j, k));
  f.saved[1][t] = p.E[q][g];
  bool in_box;
  const long long pb = pole_index(p, i, j, k, in_box);
  // f_w of E: chi1inv (D - sum of P) of the old D and of the polarization the E half
  // overwrites, as the step kernels recompute it
  float fw = p.D[q][g];
  for (int m = 0; m < p.npoles; ++m) {
    const mgb_pole& pole = p.poles[m];
    const float* prv = parity ? pole.p[q][0] : pole.p[q][1];
    const float pp = (in_box && pole.sigma[q] != nullptr) ? prv[pb] : 0.f;
    f.saved[1][(2 + m) * n + t] = pp;
    if (in_box && pole.sigma[q] != nullptr) fw = fw - pp;
  }
  f.saved[1][n + t] = sw ? __ldg(p.inv_eps[q] + g) * fw : 0.f;
}

// One B ghost: B from its image, zero_metal_B, then update_H on its own-axis membership.
__device__ __forceinline__ void fold_h_ghost(const StepParams& p, const FoldArgs& f, int t, int first_step) {
  const int n = f.count[0], g = f.ghost[0][t], r = f.image[0][t], code = f.code[0][t], q = code & 3;
  int i, j, k;
  cell_of(p, r, i, j, k);
  const bool sb_image = p.pml && in_runs(p.B[q], coord_along(q, i, j, k));
  float b = sb_image ? p.B[q].data[r] : p.H[q][r];
  if (code & 4) b = -b;
  if (code & 8) b = 0.f;
  cell_of(p, g, i, j, k);
  const int cq = coord_along(q, i, j, k);
  float h = b;
  if (p.pml && in_runs(p.B[q], cq)) {
    const float h_old = f.saved[0][t], w_old = f.saved[0][n + t];
    const float kps = ldgf(p.kps[kInteger][q], cq), kms = ldgf(p.kms[kInteger][q], cq);
    h = (first_step ? b : h_old) + (kps * b - kms * (first_step ? b : w_old));
    p.B[q].data[g] = b;
  }
  p.H[q][g] = h;
}

// One D ghost: D from its image, zero_metal_D, then update_E and update_P.
__device__ __forceinline__ void fold_e_ghost(const StepParams& p, const FoldArgs& f, int t, int parity) {
  const int n = f.count[1], g = f.ghost[1][t], r = f.image[1][t], code = f.code[1][t], q = code & 3;
  float d = p.D[q][r];
  if (code & 4) d = -d;
  if (code & 8) d = 0.f;
  p.D[q][g] = d;
  int i, j, k;
  cell_of(p, g, i, j, k);
  const int cq = coord_along(q, i, j, k);
  bool in_box;
  const long long pb = pole_index(p, i, j, k, in_box);
  float w = d;
  if (in_box)
    for (int m = 0; m < p.npoles; ++m) {
      const mgb_pole& pole = p.poles[m];
      if (pole.sigma[q] != nullptr) w = w - (parity ? pole.p[q][1] : pole.p[q][0])[pb];
    }
  w = __ldg(p.inv_eps[q] + g) * w;
  float e = w;
  if (p.pml && in_runs(p.fwE[q], cq)) {
    const float e_old = f.saved[1][t], fw_old = f.saved[1][n + t];
    e = e_old + (ldgf(p.kps[kHalf][q], cq) * w - ldgf(p.kms[kHalf][q], cq) * fw_old);
  }
  p.E[q][g] = e;
  if (in_box)
    for (int m = 0; m < p.npoles; ++m) {
      const mgb_pole& pole = p.poles[m];
      if (pole.sigma[q] == nullptr) continue;
      const float* cur = parity ? pole.p[q][1] : pole.p[q][0];
      float* prv = parity ? pole.p[q][0] : pole.p[q][1];
      const float pp = f.saved[1][(2 + m) * n + t];
      const float drive = pole.omega0dtsqr * (__ldg(pole.sigma[q] + pb) * w);
      prv[pb] = pole.gamma1inv * ((cur[pb] * pole.two_minus_od - pole.gamma1 * pp) + drive);
    }
  if (!isfinite(e) && p.status != nullptr) atomicOr(p.status, 1);
}

// After the H half: the B ghosts, and the D ghosts' state for the E half of this step
// (entries [lo, hi) of each list; thread u takes entry lo + u of both).
__global__ void __launch_bounds__(256) fold_h(const __grid_constant__ StepParams p, const __grid_constant__ FoldArgs f,
                                              int first_step, int parity) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (f.lo[0] + u < f.hi[0]) fold_h_ghost(p, f, f.lo[0] + u, first_step);
  if (f.lo[1] + u < f.hi[1]) fold_keep_e(p, f, f.lo[1] + u, parity);
}

// After the E half: the D ghosts, and the B ghosts' state for the next step's H half.
__global__ void __launch_bounds__(256) fold_e(const __grid_constant__ StepParams p, const __grid_constant__ FoldArgs f,
                                              int parity) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (f.lo[1] + u < f.hi[1]) fold_e_ghost(p, f, f.lo[1] + u, parity);
  if (f.lo[0] + u < f.hi[0]) fold_keep_h(p, f, f.lo[0] + u);
}

// The B ghosts' state, when a step is launched without the E fold of the step before.
__global__ void __launch_bounds__(256) fold_keep(const __grid_constant__ StepParams p, const __grid_constant__ FoldArgs f) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (f.lo[0] + u < f.hi[0]) fold_keep_h(p, f, f.lo[0] + u);
}

}  // namespace

// ======================================================================================
// C ABI
struct mgb_sim {
  mgb_sim_desc desc;
  StepParams step;
  TileMaps maps;
  // Kernel choice of each half (0 the H half, 1 the E half): the autotuner may pick a
  // different family and launch shape for each.
  struct HalfChoice {
    bool tiles = false;     // the tile kernels
    bool ws = false;        // the tile kernels' warp-specialized form (E half)
    bool prefetch = false;  // generic kernels: the prefetching marches
    bool l2pf = false;      // generic kernels: each thread's x chunk prefetched into L2 first
    int block_z = 32, block_y = 4, xchunk = 4;  // generic kernels
    int tile_xchunk = 8;                        // tile kernels
  } half[2];
  bool tiles_ready = false;  // their tensor maps are built
  // A D or B conductivity: the lossy generic kernels step the run (no tiles, no
  // prefetching marches, no batch slot, no adjoint).
  bool has_cond = false;
  mgb_conductivity cond = {};
  // Mirror folds: the ghost lists, and the step whose H half the B ghosts' kept state is
  // for (-1: none kept yet).
  bool folded = false;
  // step kernels of an unsplit plan launched as programmatic dependents (MEEPGB_PDL=0 at
  // mgb_create: plain launches)
  bool pdl = true;
  FoldArgs fold = {};
  long long fold_kept = -1;
  // The first entry of each x plane in each ghost list (nx + 1 entries), kept when every
  // list runs in x-plane order and every ghost's image lies in the ghost's own plane or,
  // on a folded x axis, two planes above plane 0: the x-range split then folds each
  // range's ghosts on the range's stream. Empty otherwise.
  std::vector<int> fold_plane[2];
  size_t h_smem = 0, e_smem = 0, e_ws_smem = 0;
  const double* words = nullptr;
  long long words_first = 0;
  long long words_steps = 0;
  // Monitors in buffered (tensor-core) mode: samples [kDepth][ncomp * cells], the phase
  // table scratch, and the host-tracked fill of the buffer.
  struct DftBuffer {
    float* samples = nullptr;
    float* table = nullptr;
    int count = 0;              // samples buffered since the last contraction
    long long first_post = 0;   // the step after which sample 0 was taken
  } dbuf[MGB_MAX_MONITORS];
  // The x-range split (mgb_set_split): each half launched as `ranges` launches over ranges
  // of planes on the plan's own streams, ordered by events instead of by one stream.
  struct Split {
    int ranges = 0;  // 0 or 1: off
    cudaStream_t streams[MGB_MAX_SPLIT] = {};
    cudaEvent_t h_done[2][MGB_MAX_SPLIT] = {};  // by step parity
    cudaEvent_t e_done[2][MGB_MAX_SPLIT] = {};
    cudaEvent_t fork = nullptr;
  } split;
  // The wavefront path (mgb_set_wave): runs of steps in one persistent launch.
  struct Wave {
    bool on = false;
    int bz = 32, by = 4, xchunk = 4, window = 4, max_steps = 0;
    int chunks = 0, tiles_z = 0, tiles_y = 0, blocks = 0;
    int family = 0;  // 0 the plain column marches, 2 the prefetching ones
    int l2pf = 1;    // each tile's chunk planes prefetched into L2 before its march
    unsigned* control = nullptr;
    unsigned* table = nullptr;
    unsigned* done = nullptr;
  } wave;
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

// A CUDA call that returned `err` (already taken off the sticky-free error state).
int cuda_error(cudaError_t err, const char* what) {
  cudaGetLastError();
  return fail(MGB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(err));
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (fn == nullptr) {
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult status;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault,
                                         &status) == cudaSuccess &&
        status == cudaDriverEntryPointSuccess) {
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
    }
  }
  return fn;
}

// A 3-D float32 tensor map over an (nx, ny, nz) volume with a (bz, by, 1) box.
bool make_map(CUtensorMap* map, const void* base, int nx, int ny, int nz, int bz, int by) {
  auto fn = encode_fn();
  if (fn == nullptr) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)nz, (cuuint64_t)ny, (cuuint64_t)nx};
  const cuuint64_t strides[2] = {(cuuint64_t)nz * 4, (cuuint64_t)ny * nz * 4};
  const cuuint32_t box[3] = {(cuuint32_t)bz, (cuuint32_t)by, 1};
  const cuuint32_t estride[3] = {1, 1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(base), dims,
                        strides, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Set up the tile path when the grid allows it (z rows a multiple of 16 bytes, 16-byte
// aligned volumes) and it is not switched off with MEEPGB_TILES=0.
void setup_tiles(mgb_sim* sim) {
  const char* env = getenv("MEEPGB_TILES");
  if (env != nullptr && env[0] == '0') return;
  if (sim->has_cond || sim->step.bloch || sim->step.inv) return;
  const StepParams& p = sim->step;
  if (p.nz % 4 != 0) return;
  for (int q = 0; q < 3; ++q)
    if (!aligned16(p.E[q]) || !aligned16(p.D[q]) || !aligned16(p.H[q]) || !aligned16(p.inv_eps[q]))
      return;
  TileMaps& m = sim->maps;
  memset(&m, 0, sizeof m);
  m.first_wait_ns = -1;
  bool ok = true;
  for (int q = 0; q < 3; ++q) {
    ok = ok && make_map(&m.E[q], p.E[q], p.nx, p.ny, p.nz, kHaloZ, kHaloY);
    ok = ok && make_map(&m.Hown[q], p.H[q], p.nx, p.ny, p.nz, kTileZ, kTileY);
    ok = ok && make_map(&m.Hhalo[q], p.H[q], p.nx, p.ny, p.nz, kHaloZ, kHaloY);
    ok = ok && make_map(&m.D[q], p.D[q], p.nx, p.ny, p.nz, kTileZ, kTileY);
  }
  const bool alias = p.inv_eps[0] == p.inv_eps[1] && p.inv_eps[1] == p.inv_eps[2];
  m.ninv = alias ? 1 : 3;
  for (int q = 0; q < m.ninv; ++q) ok = ok && make_map(&m.inv[q], p.inv_eps[q], p.nx, p.ny, p.nz, kTileZ, kTileY);
  for (int q = 0; q < 3; ++q) m.inv_of[q] = alias ? 0 : q;
  if (!ok) return;
  m.stages = 4;
  const char* st = getenv("MEEPGB_STAGES");
  if (st != nullptr && atoi(st) >= 2 && atoi(st) <= 8) m.stages = atoi(st);
  sim->h_smem = (size_t)m.stages * (3 * kBoxHalo + 3 * kBoxOwn) + 8 * m.stages;
  sim->e_smem = (size_t)m.stages * (3 * kBoxHalo + (3 + m.ninv) * kBoxOwn) + 8 * m.stages;
  sim->e_ws_smem = (size_t)m.stages * (3 * kBoxHalo + (3 + m.ninv) * kBoxOwn) + 16 * m.stages;
  const void* kernels[6] = {(const void*)h_tile<true>, (const void*)h_tile<false>,
                            (const void*)e_tile<true>, (const void*)e_tile<false>,
                            (const void*)e_ws<true>, (const void*)e_ws<false>};
  for (int t = 0; t < 6; ++t) {
    const size_t bytes = t < 2 ? sim->h_smem : t < 4 ? sim->e_smem : sim->e_ws_smem;
    if (cudaFuncSetAttribute(kernels[t], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) !=
        cudaSuccess) {
      cudaGetLastError();
      return;
    }
  }
  const char* xc = getenv("MEEPGB_TILE_XCHUNK");
  for (auto& h : sim->half) {
    if (xc != nullptr && atoi(xc) >= 1) h.tile_xchunk = atoi(xc);
    h.tiles = true;
  }
  sim->tiles_ready = true;
}

}  // namespace

extern "C" {

int mgb_abi_version(void) { return MGB_ABI_VERSION; }

int mgb_set_test_wait_limit(int32_t which, int64_t nanoseconds) {
  if (which < 0 || which > 1) return fail(MGB_ERR_ARGUMENT, "which must be 0 (tile stages) or 1 (contraction)");
  g_test_wait_limit[which].store(nanoseconds < 0 ? -1 : (long long)nanoseconds, std::memory_order_relaxed);
  return MGB_OK;
}

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
  if (d.nx < 1 || d.ny < 1 || d.nz < 1) return fail(MGB_ERR_ARGUMENT, "every axis needs at least one cell");
  // a one-cell axis is periodic (MEEP's unit directions; a 2-D run's invariant z): its
  // differences read the same sample twice, the exact zero of an invariant axis
  {
    const int counts[3] = {d.nx, d.ny, d.nz};
    for (int a = 0; a < 3; ++a)
      if (counts[a] == 1 && (d.metallic[a] || d.mirror[a] != 0))
        return fail(MGB_ERR_UNSUPPORTED, "an axis of one cell must be periodic (not metallic, not folded)");
    if ((d.invariant & ~7) != 0) return fail(MGB_ERR_ARGUMENT, "invariant is a bit mask of the three axes");
    for (int a = 0; a < 3; ++a)
      if (((d.invariant >> a) & 1) && (counts[a] != 1 || ((d.bloch_axes >> a) & 1)))
        return fail(MGB_ERR_ARGUMENT, "an invariant axis holds one periodic cell without a Bloch phase");
  }
  // the step kernels index a volume with 32-bit cell offsets
  if ((long long)d.nx * d.ny * d.nz >= (1LL << 31)) {
    return fail(MGB_ERR_UNSUPPORTED, "a grid of 2^31 cells or more is not stepped (32-bit cell offsets)");
  }
  const int n[3] = {d.nx, d.ny, d.nz};
  for (int q = 0; q < 3; ++q) {
    if (d.E[q] == nullptr || d.D[q] == nullptr || d.H[q] == nullptr || d.inv_eps[q] == nullptr) {
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
      if (!aux_ok(d.B[q], q, n[q], &why, "B", q) || !aux_ok(d.fwH[q], q, n[q], &why, "fwH", q) ||
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
  if (d.nsrc_magnetic < 0 || d.nsrc_magnetic > d.nsrc) {
    return fail(MGB_ERR_ARGUMENT, "nsrc_magnetic must lie in 0..nsrc");
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
      // on a periodic axis the ladder may reach one period past either face (lattice
      // images); on a folded one it may start below the plane, down to the unfolded
      // cell's low wall (mirror images)
      int lo = d.metallic[a] ? 0 : -n[a];
      int hi = d.metallic[a] ? n[a] : 2 * n[a];
      if (d.mirror[a] != 0) {
        lo = 1 - (d.full[a] - d.full[a] % 2) / 2 - (d.metallic[a] ? 0 : d.full[a]);
        hi = d.metallic[a] ? n[a] : n[a] + d.full[a];
      }
      if (mon.region[2 * a] < lo || mon.region[2 * a] >= mon.region[2 * a + 1] || mon.region[2 * a + 1] > hi) {
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
  if (d.bloch_axes & ~7) return fail(MGB_ERR_ARGUMENT, "bloch_axes holds bits 0..2 only");
  for (int a = 0; a < 3; ++a) {
    if (!((d.bloch_axes >> a) & 1)) continue;
    if (d.metallic[a]) return fail(MGB_ERR_ARGUMENT, "a Bloch phase needs a periodic axis");
    const double re = d.bloch_phase[a][0], im = d.bloch_phase[a][1];
    if (!std::isfinite(re) || !std::isfinite(im) || std::fabs(std::hypot(re, im) - 1.0) > 1e-9)
      return fail(MGB_ERR_ARGUMENT, "a Bloch phase must be a finite unit-modulus number");
  }
  if (d.bloch_axes) {
    for (int q = 0; q < 3; ++q)
      if (d.partner_E[q] == nullptr || d.partner_H[q] == nullptr)
        return fail(MGB_ERR_ARGUMENT, "a Bloch-phased plan needs the other part's E and H (partner_E, partner_H)");
  }
  bool lossy = false;
  if (d.conductivity != nullptr) {
    const mgb_conductivity& cd = *d.conductivity;
    static const char* names[2][3] = {{"Bx", "By", "Bz"}, {"Dx", "Dy", "Dz"}};
    for (int side = 0; side < 2; ++side)
      for (int q = 0; q < 3; ++q) {
        if (cd.condfac[side][q] == nullptr) continue;
        lossy = true;
        if (cd.condinv[side][q] == nullptr)
          return fail(MGB_ERR_ARGUMENT, std::string("the conductivity of ") + names[side][q] + " has no condinv volume");
        if (d.pml_active && cd.fcond[side][q] == nullptr)
          return fail(MGB_ERR_ARGUMENT, std::string("the conductivity of ") + names[side][q] +
                                            " under a PML needs its conductive-stage history (fcond)");
      }
    if (lossy && d.pml_active)
      for (int l = 0; l < 2; ++l)
        for (int a = 0; a < 3; ++a)
          if (cd.chunk_of[l][a] == nullptr)
            return fail(MGB_ERR_ARGUMENT, "a conductivity under a PML needs the chunk of every row (chunk_of)");
  }
  int fold_mask = 0;
  for (int a = 0; a < 3; ++a) {
    if (d.mirror[a] == 0) continue;
    if (d.mirror[a] != 1 && d.mirror[a] != -1)
      return fail(MGB_ERR_ARGUMENT, "a mirror phase must be +1 (even) or -1 (odd)");
    // a folded periodic axis stores one cell past MEEP's window (big_corner's plane and
    // the far ghost slot)
    const int owned = d.full[a] - d.full[a] / 2 + 1;
    if (d.full[a] < 2 || n[a] != owned + (d.metallic[a] ? 0 : 1) || n[a] < 4)
      return fail(MGB_ERR_ARGUMENT, "a folded axis stores full - full/2 + 1 cells, one more when periodic "
                                    "(at least 4)");
    fold_mask |= 1 << a;
  }
  std::vector<int> fold_plane[2];
  if (fold_mask != 0) {
    if (d.bloch_axes != 0) return fail(MGB_ERR_UNSUPPORTED, "a folded run carries no Bloch phase");
    const long long cells = (long long)n[0] * n[1] * n[2];
    for (int h = 0; h < 2; ++h) {
      const int count = d.fold.count[h];
      if (count < 0 || (count > 0 && (d.fold.ghost[h] == nullptr || d.fold.image[h] == nullptr ||
                                      d.fold.code[h] == nullptr || d.fold.saved[h] == nullptr)))
        return fail(MGB_ERR_ARGUMENT, "a mirror-fold ghost list is missing");
      if (count == 0) continue;
      // every offset inside the volume and every component 0..2, checked on the host once
      std::vector<int32_t> ghost(count), image(count);
      std::vector<uint8_t> code(count);
      if (cudaMemcpy(ghost.data(), d.fold.ghost[h], count * sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess ||
          cudaMemcpy(image.data(), d.fold.image[h], count * sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess ||
          cudaMemcpy(code.data(), d.fold.code[h], count * sizeof(uint8_t), cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return fail(MGB_ERR_ARGUMENT, "the mirror-fold ghost lists are not readable device memory");
      }
      for (int t = 0; t < count; ++t)
        if (ghost[t] < 0 || ghost[t] >= cells || image[t] < 0 || image[t] >= cells || (code[t] & 3) == 3 ||
            (code[t] & ~15) != 0)
          return fail(MGB_ERR_ARGUMENT, "a mirror-fold ghost entry lies outside the volume");
      // x-plane offsets of the list, for the x-range split
      const long long plane_cells = (long long)n[1] * n[2];
      bool ordered = true;
      for (int t = 0; t < count && ordered; ++t) {
        const int gx = (int)(ghost[t] / plane_cells), ix = (int)(image[t] / plane_cells);
        ordered = (t == 0 || ghost[t - 1] / plane_cells <= gx) && (ix == gx || (gx == 0 && ix == 2));
      }
      fold_plane[h].clear();
      if (ordered) {
        fold_plane[h].assign(n[0] + 1, count);
        for (int t = count - 1; t >= 0; --t) fold_plane[h][ghost[t] / plane_cells] = t;
        for (int x = n[0] - 1; x >= 0; --x) fold_plane[h][x] = std::min(fold_plane[h][x], fold_plane[h][x + 1]);
      }
    }
  } else if (d.fold.count[0] != 0 || d.fold.count[1] != 0) {
    return fail(MGB_ERR_ARGUMENT, "mirror-fold ghost lists without a mirror plane");
  }
  {
    // Load the kernels a run may first launch only after its first steps (the monitors'
    // samples and contractions, and a reduced-dimension run's step kernels) now: under
    // lazy module loading a first launch loads its whole module, which cost a 2-D run's
    // first timed call about 11 ms when its first sample was this module's first launch.
    cudaFuncAttributes attr;
    const void* monitors[] = {reinterpret_cast<const void*>(dft_sample), reinterpret_cast<const void*>(dft_accumulate),
                              reinterpret_cast<const void*>(flux_reduce)};
    cudaError_t err = cudaSuccess;
    for (const void* k : monitors)
      if (err == cudaSuccess) err = cudaFuncGetAttributes(&attr, k);
    if (err == cudaSuccess) err = mgbdft::preload_kernels();
    if (err == cudaSuccess && (d.invariant & 7) != 0) err = mgbred::preload_kernels();
    if (err != cudaSuccess) return cuda_error(err, "loading the monitor and step kernels");
  }
  mgb_sim* sim = new (std::nothrow) mgb_sim();
  if (sim == nullptr) return fail(MGB_ERR_ARGUMENT, "host allocation of the plan failed");
  sim->desc = d;
  sim->desc.conductivity = nullptr;  // the caller's struct need not outlive this call
  const char* pdl = getenv("MEEPGB_PDL");
  sim->pdl = !(pdl != nullptr && pdl[0] == '0');
  if (lossy) {
    sim->has_cond = true;
    sim->cond = *d.conductivity;
  }
  StepParams& p = sim->step;
  p.nx = d.nx; p.ny = d.ny; p.nz = d.nz;
  p.pml = d.pml_active ? 1 : 0;
  {
    const int n[3] = {d.nx, d.ny, d.nz};
    for (int a = 0; a < 3; ++a) {
      p.inner[2 * a] = 0;
      p.inner[2 * a + 1] = n[a];
    }
    if (p.pml) {
      const mgb_aux* families[5] = {d.B, d.fwH, d.fwE, d.fuB, d.fuD};
      for (const mgb_aux* fam : families)
        for (int q = 0; q < 3; ++q) {
          const mgb_aux& a = fam[q];
          if (a.a1 > a.a0) p.inner[2 * a.axis] = std::max(p.inner[2 * a.axis], a.a1);
          if (a.b1 > a.b0) p.inner[2 * a.axis + 1] = std::min(p.inner[2 * a.axis + 1], a.b0);
        }
    }
  }
  // a folded axis steps as a metallic one (zero words past either face, its cell 0 of
  // the shift-0 components masked and held like a wall sample until the fold writes it),
  // whatever its outer face: past a periodic one the readers are the far ghost slot,
  // which the fold writes too
  for (int a = 0; a < 3; ++a) p.met[a] = (d.metallic[a] || d.mirror[a] != 0) ? 1 : 0;
  p.inv = d.invariant & 7;
  p.dtdx = d.dtdx;
  for (int l = 0; l < 2; ++l)
    for (int a = 0; a < 3; ++a) {
      p.kms[l][a] = d.kms[l][a];
      p.sinv[l][a] = d.sinv[l][a];
      p.kps[l][a] = d.kps[l][a];
    }
  for (int q = 0; q < 3; ++q) {
    p.E[q] = d.E[q]; p.D[q] = d.D[q]; p.H[q] = d.H[q]; p.inv_eps[q] = d.inv_eps[q];
    p.B[q] = d.B[q]; p.fwH[q] = d.fwH[q]; p.fwE[q] = d.fwE[q]; p.fuB[q] = d.fuB[q]; p.fuD[q] = d.fuD[q];
  }
  p.npoles = d.npoles;
  for (int a = 0; a < 6; ++a) { p.pbox[a] = d.pbox[a]; p.src_box[a] = d.src_box[a]; }
  for (int m = 0; m < d.npoles; ++m) p.poles[m] = d.poles[m];
  p.nsrc = d.nsrc;
  p.nsrc_h = d.nsrc_magnetic;
  for (int a = 0; a < 6; ++a) p.src_box_h[a] = d.src_box_magnetic[a];
  p.src_cell = d.src_cell;
  p.src_comp = d.src_comp;
  p.src_words = nullptr;
  p.status = d.status;
  p.l2pf = 0;
  p.bloch = d.bloch_axes & 7;
  p.part = d.part ? 1 : 0;
  for (int a = 0; a < 3; ++a) {
    p.bmode[a] = 0;
    p.bre[a] = 1.f;
    p.bim[a] = 0.f;
    p.pE[a] = d.partner_E[a];
    p.pH[a] = d.partner_H[a];
    if (!((p.bloch >> a) & 1)) continue;
    const double re = d.bloch_phase[a][0], im = d.bloch_phase[a][1];
    // MEEP's connection rule: a copy within 1e-13 of +1, a negation within 1e-13 of -1
    if (std::fabs(im) < 1e-13 && std::fabs(re - 1.0) < 1e-13) p.bmode[a] = 1;
    else if (std::fabs(im) < 1e-13 && std::fabs(re + 1.0) < 1e-13) { p.bmode[a] = 2; p.bre[a] = -1.f; }
    else { p.bmode[a] = 3; p.bre[a] = (float)re; p.bim[a] = (float)im; }
  }
  if (fold_mask != 0) {
    sim->folded = true;
    for (int h = 0; h < 2; ++h) {
      sim->fold.count[h] = d.fold.count[h];
      sim->fold.ghost[h] = d.fold.ghost[h];
      sim->fold.image[h] = d.fold.image[h];
      sim->fold.code[h] = d.fold.code[h];
      sim->fold.saved[h] = d.fold.saved[h];
      sim->fold.lo[h] = 0;
      sim->fold.hi[h] = d.fold.count[h];
    }
    const bool planes_known = (d.fold.count[0] == 0 || !fold_plane[0].empty()) &&
                              (d.fold.count[1] == 0 || !fold_plane[1].empty());
    for (int h = 0; h < 2 && planes_known; ++h) {
      if (fold_plane[h].empty()) fold_plane[h].assign(n[0] + 1, 0);
      sim->fold_plane[h] = std::move(fold_plane[h]);
    }
  }
  setup_tiles(sim);
  *out = sim;
  return MGB_OK;
}

int mgb_set_launch_shape(mgb_sim* sim, int block_z, int block_y, int xchunk) {
  if (sim == nullptr) return fail(MGB_ERR_ARGUMENT, "null plan");
  if (block_z < 1 || block_y < 1 || block_z * block_y > 256 || (block_z * block_y) % 32 != 0 ||
      xchunk < 1) {
    return fail(MGB_ERR_ARGUMENT,
                "launch shape needs block_z*block_y a multiple of 32 up to 256 and x_chunk >= 1");
  }
  for (auto& h : sim->half) {
    h.block_z = block_z;
    h.block_y = block_y;
    h.xchunk = xchunk;
    h.tile_xchunk = xchunk;
  }
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

// Whether step kernels launch as programmatic dependents: in an unsplit plan the next
// half's CTAs then take the SMs the last wave of the half before frees (192^3 sphere:
// 0.1542 -> 0.1485 ms a step); across the x-range split's streams their waiting CTAs
// would hold slots the other ranges' kernels fill (0.1400 -> 0.1509), so a split plan
// launches plainly, as does a plan made with MEEPGB_PDL=0.
bool step_pdl(const mgb_sim* sim) { return sim->pdl && sim->split.ranges <= 1; }

// Launch a step kernel, as a programmatic dependent of the kernel before it in the
// stream when step_pdl (every step kernel begins with step_entry, which waits for that
// kernel before touching memory).
template <typename... KArgs, typename... Args>
void launch_step(const mgb_sim* sim, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                 Args&&... args) {
  if (!step_pdl(sim)) {
    kernel<<<grid, block, smem, s>>>(std::forward<Args>(args)...);
    return;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);  // errors: launch_error
}

// Add a monitor's buffered samples to its accumulators: one phase table and one
// contraction launch for its E components (sampled at post * dt), then the same for its
// H components (at post * dt - dt / 2). The table scratch is reused in stream order.
int flush_monitor(mgb_sim* sim, int m, cudaStream_t s) {
  mgb_sim::DftBuffer& buf = sim->dbuf[m];
  if (buf.samples == nullptr || buf.count == 0) return MGB_OK;
  const mgb_monitor& mon = sim->desc.monitors[m];
  const long long cells = (long long)(mon.region[1] - mon.region[0]) * (mon.region[3] - mon.region[2]) *
                          (mon.region[5] - mon.region[4]);
  for (int half_back = 0; half_back < 2; ++half_back) {
    mgbdft::Contraction c = {};
    c.samples = buf.samples;
    c.ld = (long long)mon.ncomp * cells;
    c.ncols = cells;
    c.nsamples = buf.count;
    c.acc = mon.acc;
    c.acc_ld = cells;
    c.nfreq = mon.nfreq;
    c.table = buf.table;
    c.status = sim->step.status;
    for (int q = 0; q < mon.ncomp; ++q) {
      if ((mon.comp[q] >= 3) != (half_back == 1)) continue;
      c.sample_off[c.ncomp] = (long long)q * cells;
      c.acc_off[c.ncomp] = (long long)q * 2 * mon.nfreq * cells;
      ++c.ncomp;
    }
    if (c.ncomp == 0) continue;
    c.first_wait_ns = test_wait_limit(1);
    const cudaError_t err =
        mgbdft::launch_contraction(mon.omega, buf.first_post, mon.decimation, mon.dt, half_back, mon.scale, c, s);
    if (err != cudaSuccess) return cuda_error(err, "tensor-core DFT contraction");
  }
  buf.count = 0;
  return MGB_OK;
}

// Launches of one step, split by part so mgb_step and mgb_launch share them.
// plane0 / plane1: the planes [plane0, plane1) a generic-kernel half covers (plane0 a
// multiple of the half's x chunk; plane1 -1 for the last plane); the tile kernels always
// cover every plane.
int launch_part_kernels(mgb_sim* sim, long long n, int part, cudaStream_t s, int plane0 = 0, int plane1 = -1) {
  StepParams& p = sim->step;
  const bool pml = sim->desc.pml_active != 0;
  if (part == 0 || part == 1) {
    if (p.nsrc > 0) p.src_words = sim->words + (n - sim->words_first) * p.nsrc;
    const mgb_sim::HalfChoice& hc = sim->half[part];
    if (hc.tiles) {
      const int xc = hc.tile_xchunk;
      const dim3 grid((p.nz + kTileZ - 1) / kTileZ, (p.ny + kTileY - 1) / kTileY,
                      (p.nx + xc - 1) / xc);
      sim->maps.first_wait_ns = test_wait_limit(0);  // the launch takes the maps by value
      if (part == 0) {
        if (pml) launch_step(sim, h_tile<true>, grid, dim3(kThreads), sim->h_smem, s, p, sim->maps, (int)(n == 0), xc);
        else launch_step(sim, h_tile<false>, grid, dim3(kThreads), sim->h_smem, s, p, sim->maps, (int)(n == 0), xc);
      } else {
        if (hc.ws) {
          if (pml) launch_step(sim, e_ws<true>, grid, dim3(kWsThreads), sim->e_ws_smem, s, p, sim->maps, (int)(n & 1), xc);
          else launch_step(sim, e_ws<false>, grid, dim3(kWsThreads), sim->e_ws_smem, s, p, sim->maps, (int)(n & 1), xc);
        } else if (pml) {
          launch_step(sim, e_tile<true>, grid, dim3(kThreads), sim->e_smem, s, p, sim->maps, (int)(n & 1), xc);
        } else {
          launch_step(sim, e_tile<false>, grid, dim3(kThreads), sim->e_smem, s, p, sim->maps, (int)(n & 1), xc);
        }
      }
      return MGB_OK;
    }
    const dim3 block(hc.block_z, hc.block_y, 1);
    const int xc = hc.xchunk;
    const int last = plane1 < 0 ? p.nx : plane1;
    const dim3 grid((p.nz + block.x - 1) / block.x, (p.ny + block.y - 1) / block.y, (last - plane0 + xc - 1) / xc);
    p.l2pf = hc.l2pf ? 1 : 0;  // per half; the launch takes the parameters by value
    p.xbase = plane0 / xc;     // ditto: the first chunk of this launch's planes
    const bool msrc = p.nsrc_h > 0;  // the H kernels with the magnetic deposit compiled in
    if (p.inv != 0) {  // a 2-D or 1-D run: its own kernels, whatever the generic family
      const cudaError_t err = mgbred::launch_half(p, sim->cond, sim->has_cond, msrc, pml, part,
                                                  part == 0 ? (int)(n == 0) : (int)(n & 1), grid, block, xc,
                                                  step_pdl(sim), s);
      if (err != cudaSuccess) return cuda_error(err, "reduced-dimension step launch");
      return MGB_OK;
    }
    if (sim->has_cond) {
      if (part == 0) {
        if (pml && msrc) launch_step(sim, h_generic_cond<true, true>, grid, block, 0, s, p, sim->cond, (int)(n == 0), xc);
        else if (pml) launch_step(sim, h_generic_cond<true, false>, grid, block, 0, s, p, sim->cond, (int)(n == 0), xc);
        else if (msrc) launch_step(sim, h_generic_cond<false, true>, grid, block, 0, s, p, sim->cond, (int)(n == 0), xc);
        else launch_step(sim, h_generic_cond<false, false>, grid, block, 0, s, p, sim->cond, (int)(n == 0), xc);
      } else {
        if (pml) launch_step(sim, e_generic_cond<true>, grid, block, 0, s, p, sim->cond, (int)(n & 1), xc);
        else launch_step(sim, e_generic_cond<false>, grid, block, 0, s, p, sim->cond, (int)(n & 1), xc);
      }
      return MGB_OK;
    }
    if (hc.prefetch) {
      if (part == 0) {
        if (pml && msrc) launch_step(sim, h_generic_pf<true, true>, grid, block, 0, s, p, (int)(n == 0), xc);
        else if (pml) launch_step(sim, h_generic_pf<true, false>, grid, block, 0, s, p, (int)(n == 0), xc);
        else if (msrc) launch_step(sim, h_generic_pf<false, true>, grid, block, 0, s, p, (int)(n == 0), xc);
        else launch_step(sim, h_generic_pf<false, false>, grid, block, 0, s, p, (int)(n == 0), xc);
      } else {
        if (pml) launch_step(sim, e_generic_pf<true>, grid, block, 0, s, p, (int)(n & 1), xc);
        else launch_step(sim, e_generic_pf<false>, grid, block, 0, s, p, (int)(n & 1), xc);
      }
    } else if (part == 0) {
      if (pml && msrc) launch_step(sim, h_generic<true, true>, grid, block, 0, s, p, (int)(n == 0), xc);
      else if (pml) launch_step(sim, h_generic<true, false>, grid, block, 0, s, p, (int)(n == 0), xc);
      else if (msrc) launch_step(sim, h_generic<false, true>, grid, block, 0, s, p, (int)(n == 0), xc);
      else launch_step(sim, h_generic<false, false>, grid, block, 0, s, p, (int)(n == 0), xc);
    } else {
      if (pml) launch_step(sim, e_generic<true>, grid, block, 0, s, p, (int)(n & 1), xc);
      else launch_step(sim, e_generic<false>, grid, block, 0, s, p, (int)(n & 1), xc);
    }
    return MGB_OK;
  }
  const long long post = n + 1;
  for (int m = 0; m < sim->desc.nmonitors; ++m) {
    const mgb_monitor& mon = sim->desc.monitors[m];
    if (post % mon.decimation != 0) continue;
    DftParams q = {};
    q.nx = p.nx; q.ny = p.ny; q.nz = p.nz;
    for (int a = 0; a < 3; ++a) q.met[a] = p.met[a];
    for (int c = 0; c < 3; ++c) { q.E[c] = p.E[c]; q.H[c] = p.H[c]; }
    q.mon = mon;
    if (sim->folded) {
      for (int a = 0; a < 3; ++a) {
        if (sim->desc.mirror[a] == 0) continue;
        q.fold |= 1 << a;
        if (!sim->desc.metallic[a]) q.far |= 1 << a;
        q.full[a] = sim->desc.full[a];
        // E/D odd about the plane normal to its own direction, H/B about the others
        for (int comp = 0; comp < 6; ++comp) {
          const bool own = comp % 3 == a;
          const int parity = (comp < 3) == own ? -sim->desc.mirror[a] : sim->desc.mirror[a];
          if (parity < 0) q.neg[comp] |= 1 << a;
        }
      }
    }
    q.bloch = p.bloch;
    q.part = p.part;
    for (int a = 0; a < 3; ++a) {
      q.bmode[a] = p.bmode[a]; q.bre[a] = p.bre[a]; q.bim[a] = p.bim[a];
      q.pE[a] = p.pE[a]; q.pH[a] = p.pH[a];
    }
    const long long cells = (long long)(mon.region[1] - mon.region[0]) *
                            (mon.region[3] - mon.region[2]) * (mon.region[5] - mon.region[4]);
    const unsigned blocks = (unsigned)((cells + 255) / 256);
    mgb_sim::DftBuffer& buf = sim->dbuf[m];
    if (buf.samples != nullptr) {
      if (buf.count == 0) buf.first_post = post;
      dft_sample<<<blocks, 256, 0, s>>>(q, buf.samples + (long long)buf.count * mon.ncomp * cells);
      if (++buf.count == mgbdft::kDepth) {
        const int rc = flush_monitor(sim, m, s);
        if (rc != MGB_OK) return rc;
      }
      continue;
    }
    const size_t smem = (size_t)mon.nfreq * 2 * sizeof(float2);
    dft_accumulate<<<blocks, 256, smem, s>>>(q, post);
  }
  return MGB_OK;
}

// One part of step n over x planes [plane0, plane1) (plane1 < 0: every plane), with the
// mirror folds of those planes' ghosts after each half of a folded run. A ranged call
// leaves the kept-state step to its caller, which sets it once every range's E half is
// queued.
int launch_part(mgb_sim* sim, long long n, int part, cudaStream_t s, int plane0 = 0, int plane1 = -1) {
  if (!sim->folded || part == 2) return launch_part_kernels(sim, n, part, s, plane0, plane1);
  FoldArgs f = sim->fold;
  if (plane1 >= 0) {
    for (int h = 0; h < 2; ++h) {
      f.lo[h] = sim->fold_plane[h][plane0];
      f.hi[h] = sim->fold_plane[h][plane1];
    }
  }
  const int c0 = f.hi[0] - f.lo[0], c1 = f.hi[1] - f.lo[1];
  const unsigned blocks = (unsigned)((std::max(c0, c1) + 255) / 256);
  if (part == 0 && sim->fold_kept != n && c0 > 0)
    fold_keep<<<(unsigned)((c0 + 255) / 256), 256, 0, s>>>(sim->step, f);
  const int rc = launch_part_kernels(sim, n, part, s, plane0, plane1);
  if (rc != MGB_OK) return rc;
  if (blocks == 0) return MGB_OK;
  if (part == 0) {
    fold_h<<<blocks, 256, 0, s>>>(sim->step, f, (int)(n == 0), (int)(n & 1));
  } else {
    fold_e<<<blocks, 256, 0, s>>>(sim->step, f, (int)(n & 1));
    if (plane1 < 0) sim->fold_kept = n + 1;
  }
  return MGB_OK;
}

// Byte layout of a wave buffer: control words, one block's table, the run's counters.
size_t wave_table_offset() { return (size_t)mgbwave::kControlWords * sizeof(unsigned); }
size_t wave_done_offset(int window, int chunks) {
  const size_t table = (size_t)mgbwave::table_entries(window, chunks) * sizeof(unsigned);
  return wave_table_offset() + ((table + 255) / 256) * 256;
}

// Steps [first, first + nsteps) on the wavefront path: runs cut after every step on which
// a monitor is due (its sample then runs between launches) and at the buffer's step limit.
int step_wave(mgb_sim* sim, long long first, int nsteps, cudaStream_t s) {
  mgb_sim::Wave& wv = sim->wave;
  const long long end = first + nsteps;
  long long n = first;
  const bool pml = sim->desc.pml_active != 0;
  const bool msrc = sim->step.nsrc_h > 0;
  while (n < end) {
    long long stop = std::min(end, n + wv.max_steps);
    for (int m = 0; m < sim->desc.nmonitors; ++m) {
      const long long dec = sim->desc.monitors[m].decimation;
      const long long due = ((n + 1 + dec - 1) / dec) * dec - 1;  // first step >= n with (step + 1) % dec == 0
      stop = std::min(stop, due + 1);
    }
    const int steps = (int)(stop - n);
    cudaError_t err = cudaMemsetAsync(wv.control, 0, wave_table_offset(), s);
    if (err == cudaSuccess) err = cudaMemsetAsync(wv.done, 0, (size_t)steps * 2 * wv.chunks * sizeof(unsigned), s);
    if (err != cudaSuccess) return cuda_error(err, "wave counters");
    mgbwave::WaveArgs w = {};
    w.control = wv.control;
    w.table = wv.table;
    w.done = wv.done;
    w.words = sim->words;
    w.words_first = sim->words_first;
    w.first = n;
    w.steps = steps;
    w.window = wv.window;
    w.chunks = wv.chunks;
    w.xchunk = wv.xchunk;
    w.tiles_z = wv.tiles_z;
    w.tiles_y = wv.tiles_y;
    const long long blocks = (steps + wv.window - 1) / wv.window;
    w.total = (unsigned long long)blocks * wv.window * 2 * wv.chunks * wv.tiles_z * wv.tiles_y;
    StepParams p = sim->step;
    p.l2pf = wv.l2pf;
    p.src_words = nullptr;
    err = mgbwave::launch_wave(p, w, wv.blocks, dim3(wv.bz, wv.by, 1), wv.family, pml, msrc, s);
    if (err != cudaSuccess) return cuda_error(err, "wavefront step launch");
    const int rc = launch_part(sim, stop - 1, 2, s);  // the monitors due after the run's last step
    if (rc != MGB_OK) return rc;
    n = stop;
  }
  return MGB_OK;
}

// Planes per range of the x-range split: a multiple of both halves' x chunks.
int split_planes(const mgb_sim* sim) {
  const int a = sim->half[0].xchunk, b = sim->half[1].xchunk;
  int g = a, h = b;
  while (h != 0) { const int t = g % h; g = h; h = t; }
  const int unit = a / g * b;
  const int per = (sim->step.nx + sim->split.ranges - 1) / sim->split.ranges;
  return ((per + unit - 1) / unit) * unit;
}

// Steps [first, first + nsteps) with each half split into x ranges on the plan's streams:
// H(n, r) after E(n-1, r) and E(n-1, r+1) (it reads E one plane above and overwrites the H
// that E(n-1, r+1) read), E(n, r) after H(n, r) and H(n, r-1) (it reads H one plane below
// and overwrites the E that H(n, r-1) read). So the GPU fills a range's tail with the next
// ready range and starts step n+1 on the low ranges while step n finishes the high ones.
// On a folded run each half of a range is followed, on the range's stream, by the fold of
// the range's ghosts (their images lie in the range: the same plane, or plane 2 for the
// ghosts of a folded x axis, which the first range holds), so the events above cover the
// ghost words too. The monitors due after a step run on the caller's stream, joined
// before and forked after; the caller's stream waits for every range at the end.
int step_split(mgb_sim* sim, long long first, int nsteps, cudaStream_t origin) {
  mgb_sim::Split& sp = sim->split;
  const int R = sp.ranges;
  const int planes = split_planes(sim);
  int ranges_used = 0;
  int lo[MGB_MAX_SPLIT], hi[MGB_MAX_SPLIT];
  for (int r = 0; r < R; ++r) {
    lo[r] = r * planes;
    hi[r] = std::min((r + 1) * planes, sim->step.nx);
    if (lo[r] < hi[r]) ranges_used = r + 1;
  }
  auto fork = [&]() -> cudaError_t {
    cudaError_t err = cudaEventRecord(sp.fork, origin);
    for (int r = 0; r < ranges_used && err == cudaSuccess; ++r) err = cudaStreamWaitEvent(sp.streams[r], sp.fork, 0);
    return err;
  };
  auto join = [&](int b) -> cudaError_t {
    cudaError_t err = cudaSuccess;
    for (int r = 0; r < ranges_used && err == cudaSuccess; ++r) err = cudaStreamWaitEvent(origin, sp.e_done[b][r], 0);
    return err;
  };
  cudaError_t err = fork();
  if (err != cudaSuccess) return cuda_error(err, "split fork");
  for (int t = 0; t < nsteps; ++t) {
    const long long n = first + t;
    const int b = (int)(n & 1), pb = b ^ 1;
    for (int r = 0; r < ranges_used; ++r) {
      if (t > 0 && r + 1 < ranges_used) {
        err = cudaStreamWaitEvent(sp.streams[r], sp.e_done[pb][r + 1], 0);
        if (err != cudaSuccess) return cuda_error(err, "split wait");
      }
      const int rc = launch_part(sim, n, 0, sp.streams[r], lo[r], hi[r]);
      if (rc != MGB_OK) return rc;
      err = cudaEventRecord(sp.h_done[b][r], sp.streams[r]);
      if (err != cudaSuccess) return cuda_error(err, "split record");
    }
    for (int r = 0; r < ranges_used; ++r) {
      if (r > 0) {
        err = cudaStreamWaitEvent(sp.streams[r], sp.h_done[b][r - 1], 0);
        if (err != cudaSuccess) return cuda_error(err, "split wait");
      }
      const int rc = launch_part(sim, n, 1, sp.streams[r], lo[r], hi[r]);
      if (rc != MGB_OK) return rc;
      err = cudaEventRecord(sp.e_done[b][r], sp.streams[r]);
      if (err != cudaSuccess) return cuda_error(err, "split record");
    }
    sim->fold_kept = n + 1;  // every range's B ghosts' state is kept for step n + 1
    bool due = false;
    for (int m = 0; m < sim->desc.nmonitors; ++m)
      if ((n + 1) % sim->desc.monitors[m].decimation == 0) due = true;
    if (due) {
      err = join(b);
      if (err != cudaSuccess) return cuda_error(err, "split join");
      const int rc = launch_part(sim, n, 2, origin);
      if (rc != MGB_OK) return rc;
      err = fork();
      if (err != cudaSuccess) return cuda_error(err, "split fork");
    }
  }
  sim->step.xbase = 0;
  err = join((int)((first + nsteps - 1) & 1));
  if (err != cudaSuccess) return cuda_error(err, "split join");
  return launch_error("split step launch");
}

void free_split(mgb_sim* sim) {
  mgb_sim::Split& sp = sim->split;
  for (int r = 0; r < MGB_MAX_SPLIT; ++r) {
    if (sp.streams[r] != nullptr) cudaStreamDestroy(sp.streams[r]);
    for (int b = 0; b < 2; ++b) {
      if (sp.h_done[b][r] != nullptr) cudaEventDestroy(sp.h_done[b][r]);
      if (sp.e_done[b][r] != nullptr) cudaEventDestroy(sp.e_done[b][r]);
    }
  }
  if (sp.fork != nullptr) cudaEventDestroy(sp.fork);
  sp = mgb_sim::Split();
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
  if (sim->wave.on) return step_wave(sim, first_step, nsteps, s);
  // (a folded x axis images plane 2 onto plane 0: the first range must hold both)
  if (sim->split.ranges > 1 && !sim->half[0].tiles && !sim->half[1].tiles &&
      (!sim->folded || sim->desc.mirror[0] == 0 || split_planes(sim) >= 3))
    return step_split(sim, first_step, nsteps, s);
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

int mgb_set_split(mgb_sim* sim, int32_t ranges) {
  if (sim == nullptr) return fail(MGB_ERR_ARGUMENT, "null plan");
  if (ranges < 0 || ranges > MGB_MAX_SPLIT)
    return fail(MGB_ERR_ARGUMENT, "ranges must be 0.." + std::to_string(MGB_MAX_SPLIT));
  if (ranges > 1 && (sim->step.bloch || !sim->desc.metallic[0]))
    return fail(MGB_ERR_UNSUPPORTED, "the x-range split steps runs without Bloch phases, on a metallic x axis");
  if (ranges > 1 && sim->folded && sim->fold_plane[0].empty())
    return fail(MGB_ERR_UNSUPPORTED, "the x-range split folds each range's ghosts: the ghost lists must run in "
                                     "x-plane order with each image in its ghost's plane (or plane 2 of a "
                                     "folded x axis)");
  free_split(sim);
  if (ranges <= 1) return MGB_OK;
  mgb_sim::Split& sp = sim->split;
  for (int r = 0; r < ranges; ++r) {
    cudaError_t err = cudaStreamCreateWithFlags(&sp.streams[r], cudaStreamNonBlocking);
    for (int b = 0; b < 2 && err == cudaSuccess; ++b) {
      err = cudaEventCreateWithFlags(&sp.h_done[b][r], cudaEventDisableTiming);
      if (err == cudaSuccess) err = cudaEventCreateWithFlags(&sp.e_done[b][r], cudaEventDisableTiming);
    }
    if (err != cudaSuccess) {
      free_split(sim);
      return cuda_error(err, "split streams");
    }
  }
  const cudaError_t err = cudaEventCreateWithFlags(&sp.fork, cudaEventDisableTiming);
  if (err != cudaSuccess) {
    free_split(sim);
    return cuda_error(err, "split streams");
  }
  sp.ranges = ranges;
  return MGB_OK;
}

size_t mgb_wave_bytes(mgb_sim* sim, int32_t x_chunk, int32_t window, int32_t max_steps) {
  if (sim == nullptr || x_chunk < 1 || window < 1 || window > mgbwave::kMaxWindow || max_steps < 1) return 0;
  const int chunks = (sim->step.nx + x_chunk - 1) / x_chunk;
  return wave_done_offset(window, chunks) + (size_t)max_steps * 2 * chunks * sizeof(unsigned);
}

int mgb_set_wave(mgb_sim* sim, int32_t family, int32_t block_z, int32_t block_y, int32_t x_chunk, int32_t window,
                 int32_t max_steps, void* buffer, size_t bytes, void* stream) {
  if (sim == nullptr) return fail(MGB_ERR_ARGUMENT, "null plan");
  if (buffer == nullptr) {
    sim->wave.on = false;
    return MGB_OK;
  }
  if (sim->folded || sim->step.bloch || sim->has_cond)
    return fail(MGB_ERR_UNSUPPORTED, "the wavefront path steps runs without mirror folds, Bloch phases or a "
                                     "conductivity");
  if (sim->step.inv != 0)
    return fail(MGB_ERR_UNSUPPORTED, "the wavefront path steps 3-D runs");
  if (!sim->desc.metallic[0])
    return fail(MGB_ERR_UNSUPPORTED, "the wavefront path needs a metallic x axis (a periodic x would make the "
                                     "first chunk wait on the last)");
  if (family != 0 && family != 2) return fail(MGB_ERR_ARGUMENT, "the wavefront marches are family 0 or 2");
  if (block_z < 32 || block_z % 32 != 0 || block_y < 1 || block_z * block_y > 256)
    return fail(MGB_ERR_ARGUMENT, "block_z must be a multiple of 32 and block_z * block_y at most 256");
  const size_t need = mgb_wave_bytes(sim, x_chunk, window, max_steps);
  if (need == 0) return fail(MGB_ERR_ARGUMENT, "bad x_chunk, window (1.." + std::to_string(mgbwave::kMaxWindow) +
                                                ") or max_steps");
  if (bytes < need) return fail(MGB_ERR_ARGUMENT, "wave buffer smaller than mgb_wave_bytes()");
  if ((reinterpret_cast<uintptr_t>(buffer) & 255u) != 0) return fail(MGB_ERR_ARGUMENT, "wave buffer not 256-byte aligned");
  const int chunks = (sim->step.nx + x_chunk - 1) / x_chunk;
  if (chunks >= (1 << 16)) return fail(MGB_ERR_ARGUMENT, "too many x chunks for the item table");
  const bool pml = sim->desc.pml_active != 0;
  const bool msrc = sim->step.nsrc_h > 0;
  const int per_sm = mgbwave::wave_blocks_per_sm(block_z * block_y, family, pml, msrc);
  int device = 0, sms = 0;
  if (per_sm <= 0 || cudaGetDevice(&device) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return launch_error("wavefront occupancy");
  mgb_sim::Wave& wv = sim->wave;
  unsigned char* base = static_cast<unsigned char*>(buffer);
  wv.family = family;
  const char* l2pf = getenv("MEEPGB_WAVE_L2PF");
  wv.l2pf = (l2pf != nullptr && l2pf[0] == '0') ? 0 : 1;
  wv.bz = block_z;
  wv.by = block_y;
  wv.xchunk = x_chunk;
  wv.window = window;
  wv.max_steps = max_steps;
  wv.chunks = chunks;
  wv.tiles_z = (sim->step.nz + block_z - 1) / block_z;
  wv.tiles_y = (sim->step.ny + block_y - 1) / block_y;
  wv.blocks = per_sm * sms;
  wv.control = reinterpret_cast<unsigned*>(base);
  wv.table = reinterpret_cast<unsigned*>(base + wave_table_offset());
  wv.done = reinterpret_cast<unsigned*>(base + wave_done_offset(window, chunks));
  const cudaError_t err = mgbwave::launch_wave_table(wv.table, window, chunks, static_cast<cudaStream_t>(stream));
  if (err != cudaSuccess) return cuda_error(err, "wave table");
  wv.on = true;
  return MGB_OK;
}

int mgb_step_pair(mgb_sim* real, mgb_sim* imag, int64_t first_step, int32_t nsteps, void* stream) {
  if (real == nullptr || imag == nullptr) return fail(MGB_ERR_ARGUMENT, "null plan");
  if (real->step.part != 0 || imag->step.part != 1)
    return fail(MGB_ERR_ARGUMENT, "mgb_step_pair takes the real-part plan, then the imaginary-part plan");
  if (nsteps < 0 || first_step < 0) return fail(MGB_ERR_ARGUMENT, "negative step range");
  if (nsteps == 0) return MGB_OK;
  int rc = check_words(real, first_step, nsteps);
  if (rc == MGB_OK) rc = check_words(imag, first_step, nsteps);
  if (rc != MGB_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  for (int32_t t = 0; t < nsteps; ++t) {
    const long long n = first_step + t;
    for (int part = 0; part < 3; ++part) {
      launch_part(real, n, part, s);
      launch_part(imag, n, part, s);
    }
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
  const int rc = flush_monitor(sim, monitor, static_cast<cudaStream_t>(stream));
  if (rc != MGB_OK) return rc;
  flux_reduce<<<m.nfreq, 256, 0, static_cast<cudaStream_t>(stream)>>>(m, weights, out);
  return launch_error("flux reduction launch");
}

int mgb_set_dft_buffer(mgb_sim* sim, int32_t monitor, float* samples, void* scratch, size_t scratch_bytes) {
  if (sim == nullptr) return fail(MGB_ERR_ARGUMENT, "null plan");
  if (monitor < 0 || monitor >= sim->desc.nmonitors) return fail(MGB_ERR_ARGUMENT, "no such monitor");
  mgb_sim::DftBuffer& buf = sim->dbuf[monitor];
  if (buf.count != 0) return fail(MGB_ERR_ARGUMENT, "the monitor holds buffered samples: mgb_dft_flush first");
  if (samples == nullptr) {
    buf = mgb_sim::DftBuffer{};
    return MGB_OK;
  }
  const mgb_monitor& m = sim->desc.monitors[monitor];
  if (m.nfreq > mgbdft::kMaxFreq || m.ncomp > mgbdft::kMaxComps)
    return fail(MGB_ERR_UNSUPPORTED, "tensor-core accumulation takes at most " + std::to_string(mgbdft::kMaxFreq) +
                                         " frequencies");
  if (scratch == nullptr || scratch_bytes < mgbdft::table_bytes(m.nfreq))
    return fail(MGB_ERR_ARGUMENT, "scratch is smaller than mgb_dft_scratch_bytes(nfreq)");
  if ((reinterpret_cast<uintptr_t>(samples) & 15u) != 0 || (reinterpret_cast<uintptr_t>(scratch) & 15u) != 0)
    return fail(MGB_ERR_ARGUMENT, "sample buffer and scratch must be 16-byte aligned");
  buf.samples = samples;
  buf.table = static_cast<float*>(scratch);
  buf.count = 0;
  return MGB_OK;
}

int mgb_dft_flush(mgb_sim* sim, void* stream) {
  if (sim == nullptr) return fail(MGB_ERR_ARGUMENT, "null plan");
  for (int m = 0; m < sim->desc.nmonitors; ++m) {
    const int rc = flush_monitor(sim, m, static_cast<cudaStream_t>(stream));
    if (rc != MGB_OK) return rc;
  }
  return MGB_OK;
}

int mgb_read_accumulator(mgb_sim* real, mgb_sim* imag, int32_t monitor, int32_t comp, float* dst,
                         void* stream) {
  if (real == nullptr || dst == nullptr) return fail(MGB_ERR_ARGUMENT, "null plan or destination");
  if (monitor < 0 || monitor >= real->desc.nmonitors) return fail(MGB_ERR_ARGUMENT, "no such monitor");
  const mgb_monitor& m = real->desc.monitors[monitor];
  if (comp < 0 || comp >= m.ncomp) return fail(MGB_ERR_ARGUMENT, "no such monitor component");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long cells = (long long)(m.region[1] - m.region[0]) * (m.region[3] - m.region[2]) *
                          (m.region[5] - m.region[4]);
  const long long nf = m.nfreq;
  const float* b = nullptr;
  int rc = flush_monitor(real, monitor, s);
  if (rc != MGB_OK) return rc;
  if (imag != nullptr) {
    if (monitor >= imag->desc.nmonitors) return fail(MGB_ERR_ARGUMENT, "the imaginary plan lacks the monitor");
    const mgb_monitor& mi = imag->desc.monitors[monitor];
    if (mi.nfreq != m.nfreq || mi.ncomp != m.ncomp || memcmp(mi.region, m.region, sizeof m.region) != 0)
      return fail(MGB_ERR_ARGUMENT, "the two plans' monitors differ");
    rc = flush_monitor(imag, monitor, s);
    if (rc != MGB_OK) return rc;
    b = mi.acc + (long long)comp * nf * 2 * cells;
  }
  const long long n = nf * cells;
  if (n == 0) return MGB_OK;
  interleave_accumulator<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(m.acc + (long long)comp * nf * 2 * cells, b,
                                                                    nf, cells, reinterpret_cast<float2*>(dst));
  return launch_error("accumulator read");
}

int32_t mgb_dft_pending(mgb_sim* sim, int32_t monitor) {
  if (sim == nullptr || monitor < 0 || monitor >= sim->desc.nmonitors) return -1;
  return sim->dbuf[monitor].count;
}

int mgb_uses_tiles(mgb_sim* sim) {
  return sim != nullptr && (sim->half[0].tiles || sim->half[1].tiles) ? 1 : 0;
}

namespace {
int choose_family(mgb_sim* sim, mgb_sim::HalfChoice& h, int family, int part) {
  if (sim->has_cond && family != 0 && family != 4)
    return fail(MGB_ERR_UNSUPPORTED, "a run with a conductivity steps with the generic kernels (family 0 or 4)");
  if (sim->step.bloch && family != 0 && family != 4)
    return fail(MGB_ERR_UNSUPPORTED, "a Bloch-phased run steps with the generic kernels (family 0 or 4)");
  if (sim->step.inv && (family == 1 || family == 3))
    return fail(MGB_ERR_UNSUPPORTED, "a reduced-dimension run steps with the generic kernel families (0, 2, 4, 5)");
  if (family == 0 || family == 2 || family == 4 || family == 5) {
    h.tiles = false;
    h.ws = false;
    h.prefetch = family == 2 || family == 5;
    h.l2pf = family == 4 || family == 5;
    return MGB_OK;
  }
  if (family == 1 || family == 3) {
    if (!sim->tiles_ready) return fail(MGB_ERR_UNSUPPORTED, "the tile kernels need a z extent that is a multiple of 4");
    if (family == 3 && part != 1) return fail(MGB_ERR_UNSUPPORTED, "the warp-specialized tile kernel steps the E half");
    h.tiles = true;
    h.ws = family == 3;
    h.prefetch = false;
    h.l2pf = false;
    return MGB_OK;
  }
  return fail(MGB_ERR_ARGUMENT,
              "kernel family is 0 (generic), 1 (tiles), 2 (generic, prefetching), 3 (tiles, warp-specialized), "
              "4 (generic, x chunk prefetched into L2) or 5 (prefetching, x chunk prefetched into L2)");
}
}  // namespace

int mgb_select_kernels(mgb_sim* sim, int32_t family) {
  if (sim == nullptr) return fail(MGB_ERR_ARGUMENT, "null plan");
  if (family == 3) return fail(MGB_ERR_UNSUPPORTED, "the warp-specialized tile kernel steps the E half only");
  for (int part = 0; part < 2; ++part) {
    const int rc = choose_family(sim, sim->half[part], family, part);
    if (rc != MGB_OK) return rc;
  }
  return MGB_OK;
}

int mgb_select_half(mgb_sim* sim, int32_t part, int32_t family, int32_t block_z, int32_t block_y,
                    int32_t x_chunk) {
  if (sim == nullptr) return fail(MGB_ERR_ARGUMENT, "null plan");
  if (part != 0 && part != 1) return fail(MGB_ERR_ARGUMENT, "part is 0 (H half) or 1 (E half)");
  if (block_z < 1 || block_y < 1 || block_z * block_y > 256 || (block_z * block_y) % 32 != 0 || x_chunk < 1)
    return fail(MGB_ERR_ARGUMENT, "launch shape needs block_z*block_y a multiple of 32 up to 256 and x_chunk >= 1");
  mgb_sim::HalfChoice h = sim->half[part];
  const int rc = choose_family(sim, h, family, part);
  if (rc != MGB_OK) return rc;
  h.block_z = block_z;
  h.block_y = block_y;
  h.xchunk = x_chunk;
  h.tile_xchunk = x_chunk;
  sim->half[part] = h;
  return MGB_OK;
}

void mgb_destroy(mgb_sim* sim) {
  if (sim == nullptr) return;
  free_split(sim);
  delete sim;
}

}  // extern "C"

// ======================================================================================
// Batched stepping ABI
struct mgb_batch {
  int max_slots = 0, max_work = 0, max_dft_work = 0;
  int block_z = 32, block_y = 4;
  int family = 2;  // the marches the step items run: 2 prefetching, 4 generic with L2 prefetch
  BatchTables dev = {};
  std::vector<StepParams> params;
  std::vector<SlotState> state;
  std::vector<long long> n0;  // each slot's next step (host-tracked)
  std::vector<DftParams> dft;
  std::vector<unsigned char> dirty;
  std::vector<int4> work, dwork;
  int nwork = 0, ndwork = 0;
  bool work_dirty = true;
  cudaGraphExec_t graph = nullptr;
  cudaGraph_t graph_src = nullptr;          // kept: its kernel nodes are updated in place
  std::vector<cudaGraphNode_t> step_nodes;  // H and E launches of every captured step
  std::vector<cudaGraphNode_t> dft_nodes;
  int graph_steps = 0;
  int graph_shape[3] = {0, 0, 0};
  int graph_grid[2] = {0, 0};
  cudaStream_t graph_stream = nullptr;
};

namespace {

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

void batch_layout(int max_slots, int max_work, int max_dft_work, size_t offsets[7], size_t* total) {
  size_t o = 0;
  offsets[0] = o; o = align256(o + sizeof(StepParams) * max_slots);
  offsets[1] = o; o = align256(o + sizeof(SlotState) * max_slots);
  offsets[2] = o; o = align256(o + sizeof(long long) * max_slots);
  offsets[3] = o; o = align256(o + sizeof(DftParams) * max_slots * kSlotMonitors);
  offsets[4] = o; o = align256(o + sizeof(int4) * max_work);
  offsets[5] = o; o = align256(o + sizeof(int4) * max_dft_work);
  offsets[6] = o; o = align256(o + sizeof(int) * 2);
  *total = o;
}

long long monitor_cells(const mgb_monitor& mon) {
  return (long long)(mon.region[1] - mon.region[0]) * (mon.region[3] - mon.region[2]) *
         (mon.region[5] - mon.region[4]);
}

void rebuild_work(mgb_batch* b) {
  b->work.clear();
  b->dwork.clear();
  const int bz = b->block_z, by = b->block_y, xc = b->dev.xchunk;
  for (int sl = 0; sl < b->max_slots; ++sl) {
    const SlotState& st = b->state[sl];
    if (!st.active) continue;
    const StepParams& p = b->params[sl];
    const int tz = (p.nz + bz - 1) / bz, ty = (p.ny + by - 1) / by, tx = (p.nx + xc - 1) / xc;
    for (int x = 0; x < tx; ++x)
      for (int y = 0; y < ty; ++y)
        for (int z = 0; z < tz; ++z) b->work.push_back(make_int4(sl, z, y, x));
    for (int m = 0; m < st.nmon; ++m) {
      const int blocks = (int)((monitor_cells(b->dft[sl * kSlotMonitors + m].mon) + kDftItemCells - 1) /
                               kDftItemCells);
      for (int q = 0; q < blocks; ++q) b->dwork.push_back(make_int4(sl * kSlotMonitors + m, q, 0, 0));
    }
  }
}

// One CTA per item (at least one, so an empty list still launches validly).
int step_grid(const mgb_batch* b) { return std::max(1, b->nwork); }
int dft_grid(const mgb_batch* b) { return std::max(1, b->ndwork); }

void batch_launch_step(mgb_batch* b, int t, cudaStream_t s) {
  const dim3 block(b->block_z, b->block_y, 1);
  if (b->family == 4) {
    step_batched<0, true><<<step_grid(b), block, 0, s>>>(b->dev, t);
    step_batched<1, true><<<step_grid(b), block, 0, s>>>(b->dev, t);
  } else {
    step_batched<0, false><<<step_grid(b), block, 0, s>>>(b->dev, t);
    step_batched<1, false><<<step_grid(b), block, 0, s>>>(b->dev, t);
  }
  dft_batched<<<dft_grid(b), kDftItemCells, 0, s>>>(b->dev, t);
}

void drop_graph(mgb_batch* b) {
  if (b->graph != nullptr) cudaGraphExecDestroy(b->graph);
  if (b->graph_src != nullptr) cudaGraphDestroy(b->graph_src);
  b->graph = nullptr;
  b->graph_src = nullptr;
  b->step_nodes.clear();
  b->dft_nodes.clear();
}

// Point the captured launches at the current list lengths (grid sizes only).
int update_graph_grids(mgb_batch* b) {
  const int grids[2] = {step_grid(b), dft_grid(b)};
  if (grids[0] == b->graph_grid[0] && grids[1] == b->graph_grid[1]) return MGB_OK;
  for (int which = 0; which < 2; ++which) {
    for (cudaGraphNode_t node : which == 0 ? b->step_nodes : b->dft_nodes) {
      cudaKernelNodeParams kp;
      if (cudaGraphKernelNodeGetParams(node, &kp) != cudaSuccess) return launch_error("graph node params");
      kp.gridDim = dim3(grids[which], 1, 1);
      if (cudaGraphExecKernelNodeSetParams(b->graph, node, &kp) != cudaSuccess)
        return launch_error("graph node update");
    }
  }
  b->graph_grid[0] = grids[0];
  b->graph_grid[1] = grids[1];
  return MGB_OK;
}

int capture_graph(mgb_batch* b, int nsteps, cudaStream_t s) {
  drop_graph(b);
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return launch_error("batch graph capture");
  for (int t = 0; t < nsteps; ++t) batch_launch_step(b, t, s);
  if (cudaStreamEndCapture(s, &b->graph_src) != cudaSuccess) {
    b->graph_src = nullptr;
    return launch_error("batch graph capture end");
  }
  const cudaError_t err = cudaGraphInstantiate(&b->graph, b->graph_src, 0);
  if (err != cudaSuccess) {
    b->graph = nullptr;
    drop_graph(b);
    return fail(MGB_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(err));
  }
  size_t count = 0;
  cudaGraphGetNodes(b->graph_src, nullptr, &count);
  std::vector<cudaGraphNode_t> nodes(count);
  if (count > 0) cudaGraphGetNodes(b->graph_src, nodes.data(), &count);
  const bool gen = b->family == 4;
  const void* h_fn = gen ? reinterpret_cast<const void*>(step_batched<0, true>)
                         : reinterpret_cast<const void*>(step_batched<0, false>);
  const void* e_fn = gen ? reinterpret_cast<const void*>(step_batched<1, true>)
                         : reinterpret_cast<const void*>(step_batched<1, false>);
  const void* d_fn = reinterpret_cast<const void*>(dft_batched);
  for (cudaGraphNode_t node : nodes) {
    cudaGraphNodeType type;
    if (cudaGraphNodeGetType(node, &type) != cudaSuccess || type != cudaGraphNodeTypeKernel) continue;
    cudaKernelNodeParams kp;
    if (cudaGraphKernelNodeGetParams(node, &kp) != cudaSuccess) continue;
    if (kp.func == h_fn || kp.func == e_fn) b->step_nodes.push_back(node);
    else if (kp.func == d_fn) b->dft_nodes.push_back(node);
  }
  if ((int)b->step_nodes.size() != 2 * nsteps || (int)b->dft_nodes.size() != nsteps) {
    drop_graph(b);
    return fail(MGB_ERR_CUDA, "captured batch graph does not hold the expected launches");
  }
  b->graph_steps = nsteps;
  b->graph_stream = s;
  b->graph_shape[0] = b->block_z;
  b->graph_shape[1] = b->block_y;
  b->graph_shape[2] = b->dev.xchunk;
  b->graph_grid[0] = step_grid(b);
  b->graph_grid[1] = dft_grid(b);
  return MGB_OK;
}

}  // namespace

extern "C" {

size_t mgb_batch_bytes(int32_t max_slots, int32_t max_work, int32_t max_dft_work) {
  size_t offsets[7], total;
  batch_layout(max_slots, max_work, max_dft_work, offsets, &total);
  return total;
}

int mgb_batch_create(int32_t max_slots, int32_t max_work, int32_t max_dft_work, void* device_buffer,
                     size_t bytes, mgb_batch** out) {
  if (out == nullptr) return fail(MGB_ERR_ARGUMENT, "null output handle");
  *out = nullptr;
  if (device_buffer == nullptr || max_slots < 1 || max_work < 1 || max_dft_work < 1)
    return fail(MGB_ERR_ARGUMENT, "a batch needs slots, work capacities and a device buffer");
  size_t offsets[7], total;
  batch_layout(max_slots, max_work, max_dft_work, offsets, &total);
  if (bytes < total) return fail(MGB_ERR_ARGUMENT, "batch device buffer is smaller than mgb_batch_bytes()");
  if ((reinterpret_cast<uintptr_t>(device_buffer) & 255u) != 0)
    return fail(MGB_ERR_ARGUMENT, "batch device buffer must be 256-byte aligned");
  mgb_batch* b = new (std::nothrow) mgb_batch();
  if (b == nullptr) return fail(MGB_ERR_ARGUMENT, "host allocation of the batch failed");
  unsigned char* base = static_cast<unsigned char*>(device_buffer);
  b->max_slots = max_slots;
  b->max_work = max_work;
  b->max_dft_work = max_dft_work;
  b->dev.params = reinterpret_cast<StepParams*>(base + offsets[0]);
  b->dev.state = reinterpret_cast<SlotState*>(base + offsets[1]);
  b->dev.n0 = reinterpret_cast<long long*>(base + offsets[2]);
  b->dev.dft = reinterpret_cast<DftParams*>(base + offsets[3]);
  b->dev.work = reinterpret_cast<int4*>(base + offsets[4]);
  b->dev.dft_work = reinterpret_cast<int4*>(base + offsets[5]);
  b->dev.counts = reinterpret_cast<int*>(base + offsets[6]);
  b->dev.max_slots = max_slots;
  b->dev.xchunk = 4;
  b->params.assign(max_slots, StepParams{});
  b->state.assign(max_slots, SlotState{});
  b->n0.assign(max_slots, 0);
  b->dft.assign((size_t)max_slots * kSlotMonitors, DftParams{});
  b->dirty.assign(max_slots, 1);
  *out = b;
  return MGB_OK;
}

int mgb_batch_set_shape(mgb_batch* b, int32_t block_z, int32_t block_y, int32_t x_chunk) {
  if (b == nullptr) return fail(MGB_ERR_ARGUMENT, "null batch");
  if (block_z < 1 || block_y < 1 || x_chunk < 1 || block_z * block_y > 256 || block_z % 32 != 0)
    return fail(MGB_ERR_ARGUMENT, "batch shape needs block_z a multiple of 32, block_z*block_y <= 256");
  b->block_z = block_z;
  b->block_y = block_y;
  b->dev.xchunk = x_chunk;
  b->work_dirty = true;
  return MGB_OK;
}

int mgb_batch_set_family(mgb_batch* b, int32_t family) {
  if (b == nullptr) return fail(MGB_ERR_ARGUMENT, "null batch");
  if (family != 2 && family != 4)
    return fail(MGB_ERR_ARGUMENT,
                "a batch steps with family 2 (prefetching marches) or 4 (generic marches, x chunk prefetched "
                "into L2)");
  if (family != b->family) {
    b->family = family;
    drop_graph(b);  // the captured launches name the other kernels
  }
  return MGB_OK;
}

int mgb_batch_set_slot(mgb_batch* b, int32_t slot, mgb_sim* sim, int64_t end_step, const double* words) {
  if (b == nullptr || sim == nullptr) return fail(MGB_ERR_ARGUMENT, "null batch or plan");
  if (slot < 0 || slot >= b->max_slots) return fail(MGB_ERR_ARGUMENT, "slot out of range");
  if (end_step < 1) return fail(MGB_ERR_ARGUMENT, "a slot needs at least one step");
  if (sim->step.nsrc > 0 && words == nullptr) return fail(MGB_ERR_ARGUMENT, "the slot's sources need deposit words");
  if (sim->has_cond) return fail(MGB_ERR_UNSUPPORTED, "a batched slot does not carry a conductivity");
  if (sim->folded) return fail(MGB_ERR_UNSUPPORTED, "a batched slot does not carry mirror folds");
  if (sim->step.inv) return fail(MGB_ERR_UNSUPPORTED, "a batched slot is a 3-D run");
  if (sim->desc.nmonitors > kSlotMonitors)
    return fail(MGB_ERR_UNSUPPORTED, "a batched slot holds at most " + std::to_string(kSlotMonitors) + " monitors");
  for (int m = 0; m < sim->desc.nmonitors; ++m) {
    if (sim->desc.monitors[m].decimation < 1) return fail(MGB_ERR_ARGUMENT, "monitor decimation must be >= 1");
    if (sim->desc.monitors[m].nfreq > kBatchMaxFreq)
      return fail(MGB_ERR_UNSUPPORTED, "a batched monitor holds at most " + std::to_string(kBatchMaxFreq) +
                                           " frequencies");
  }
  b->params[slot] = sim->step;
  b->params[slot].src_words = nullptr;
  b->params[slot].l2pf = 0;  // the batch kernel sets it from the batch's family
  SlotState st = {};
  st.end = end_step;
  st.words = words;
  st.active = 1;
  st.nmon = sim->desc.nmonitors;
  b->state[slot] = st;
  b->n0[slot] = 0;
  for (int m = 0; m < sim->desc.nmonitors; ++m) {
    DftParams& q = b->dft[slot * kSlotMonitors + m];
    q.nx = sim->step.nx; q.ny = sim->step.ny; q.nz = sim->step.nz;
    for (int a = 0; a < 3; ++a) q.met[a] = sim->step.met[a];
    for (int c = 0; c < 3; ++c) { q.E[c] = sim->step.E[c]; q.H[c] = sim->step.H[c]; }
    q.mon = sim->desc.monitors[m];
    q.bloch = sim->step.bloch;
    q.part = sim->step.part;
    for (int a = 0; a < 3; ++a) {
      q.bmode[a] = sim->step.bmode[a]; q.bre[a] = sim->step.bre[a]; q.bim[a] = sim->step.bim[a];
      q.pE[a] = sim->step.pE[a]; q.pH[a] = sim->step.pH[a];
    }
  }
  b->dirty[slot] = 1;
  b->work_dirty = true;
  return MGB_OK;
}

int mgb_batch_clear_slot(mgb_batch* b, int32_t slot) {
  if (b == nullptr) return fail(MGB_ERR_ARGUMENT, "null batch");
  if (slot < 0 || slot >= b->max_slots) return fail(MGB_ERR_ARGUMENT, "slot out of range");
  b->state[slot] = SlotState{};
  b->n0[slot] = 0;
  b->dirty[slot] = 1;
  b->work_dirty = true;
  return MGB_OK;
}

int mgb_batch_commit(mgb_batch* b, void* stream) {
  if (b == nullptr) return fail(MGB_ERR_ARGUMENT, "null batch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (b->work_dirty) {
    rebuild_work(b);
    if ((int)b->work.size() > b->max_work || (int)b->dwork.size() > b->max_dft_work)
      return fail(MGB_ERR_RANGE, "the admitted slots need " + std::to_string(b->work.size()) + " step and " +
                                     std::to_string(b->dwork.size()) + " monitor items; the batch holds " +
                                     std::to_string(b->max_work) + " and " + std::to_string(b->max_dft_work));
  }
  // Pageable host sources: each copy is staged before the call returns, so the host
  // vectors may change afterwards. Stream order puts them after the steps queued before.
  for (int sl = 0; sl < b->max_slots; ++sl) {
    if (!b->dirty[sl]) continue;
    cudaMemcpyAsync(b->dev.params + sl, &b->params[sl], sizeof(StepParams), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(b->dev.state + sl, &b->state[sl], sizeof(SlotState), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(b->dev.dft + (size_t)sl * kSlotMonitors, &b->dft[(size_t)sl * kSlotMonitors],
                    sizeof(DftParams) * kSlotMonitors, cudaMemcpyHostToDevice, s);
    b->dirty[sl] = 0;
  }
  if (b->work_dirty) {
    b->nwork = (int)b->work.size();
    b->ndwork = (int)b->dwork.size();
    if (b->nwork > 0)
      cudaMemcpyAsync(b->dev.work, b->work.data(), sizeof(int4) * b->nwork, cudaMemcpyHostToDevice, s);
    if (b->ndwork > 0)
      cudaMemcpyAsync(b->dev.dft_work, b->dwork.data(), sizeof(int4) * b->ndwork, cudaMemcpyHostToDevice, s);
    const int counts[2] = {b->nwork, b->ndwork};
    cudaMemcpyAsync(b->dev.counts, counts, sizeof counts, cudaMemcpyHostToDevice, s);
    b->work_dirty = false;
  }
  return launch_error("batch commit");
}

int mgb_batch_step(mgb_batch* b, int32_t nsteps, int32_t use_graph, void* stream) {
  if (b == nullptr || nsteps < 0) return fail(MGB_ERR_ARGUMENT, "bad batch step");
  if (b->work_dirty) return fail(MGB_ERR_ARGUMENT, "slots changed since the last mgb_batch_commit");
  if (nsteps == 0) return MGB_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // Each slot's step at the first launch (staged copy: the host vector advances below).
  cudaMemcpyAsync(b->dev.n0, b->n0.data(), sizeof(long long) * b->max_slots, cudaMemcpyHostToDevice, s);
  if (!use_graph) {
    for (int t = 0; t < nsteps; ++t) batch_launch_step(b, t, s);
    const int rc = launch_error("batch step");
    if (rc != MGB_OK) return rc;
  } else {
    const bool same = b->graph != nullptr && b->graph_steps == nsteps && b->graph_stream == s &&
                      b->graph_shape[0] == b->block_z && b->graph_shape[1] == b->block_y &&
                      b->graph_shape[2] == b->dev.xchunk;
    if (!same) {
      const int rc = capture_graph(b, nsteps, s);
      if (rc != MGB_OK) return rc;
    }
    const int rc = update_graph_grids(b);
    if (rc != MGB_OK) return rc;
    if (cudaGraphLaunch(b->graph, s) != cudaSuccess) return launch_error("batch graph launch");
  }
  for (int sl = 0; sl < b->max_slots; ++sl)
    if (b->state[sl].active) b->n0[sl] = std::min<long long>(b->state[sl].end, b->n0[sl] + nsteps);
  return MGB_OK;
}

int mgb_batch_steps(mgb_batch* b, int64_t* steps) {
  if (b == nullptr || steps == nullptr) return fail(MGB_ERR_ARGUMENT, "null argument");
  for (int sl = 0; sl < b->max_slots; ++sl) steps[sl] = b->state[sl].active ? b->n0[sl] : -1;
  return MGB_OK;
}

int64_t mgb_batch_items(mgb_batch* b, int32_t which) {
  if (b == nullptr) return -1;
  return which == 0 ? b->nwork : b->ndwork;
}

void mgb_batch_destroy(mgb_batch* b) {
  if (b == nullptr) return;
  drop_graph(b);
  delete b;
}

}  // extern "C"

// ======================================================================================
// Tensor-core DFT contraction ABI
//
// The standalone contractions (mgb_dft_contract and its allocation-free twin) report a
// tensor-core wait that ran out in a status word of the library: a file-scope device int
// beside the allocation-free entry point's phase table, so neither entry point needs a
// caller buffer for it. Both device addresses are looked up once per device
// (cudaGetSymbolAddress with that device current) and cached. The status word is sticky
// until mgb_dft_contract_status clears it.
namespace {

static __device__ __align__(256) float g_dft_table[mgbdft::kMaxTableBytes / sizeof(float)];
static __device__ int g_contract_status;

struct StaticWords {
  void* table = nullptr;
  int* status = nullptr;
};

std::mutex g_static_mutex;
std::vector<StaticWords> g_static_words;  // per device, empty until looked up

int static_words(StaticWords* out) {
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return launch_error("current device");
  std::lock_guard<std::mutex> lock(g_static_mutex);
  if ((int)g_static_words.size() <= device) g_static_words.resize(device + 1);
  StaticWords& words = g_static_words[device];
  if (words.table == nullptr) {
    void* table = nullptr;
    void* status = nullptr;
    cudaError_t err = cudaGetSymbolAddress(&table, g_dft_table);
    if (err != cudaSuccess) return cuda_error(err, "static DFT table address");
    err = cudaGetSymbolAddress(&status, g_contract_status);
    if (err != cudaSuccess) return cuda_error(err, "contraction status address");
    words.table = table;
    words.status = static_cast<int*>(status);
  }
  *out = words;
  return MGB_OK;
}

// Arguments every contraction entry point checks before it touches the device; returns
// MGB_OK, or the refusal. *nothing is set when the call has no work.
int check_contract(const float* samples, int64_t ld, int64_t ncols, int32_t nsamples, const double* omega,
                   int32_t nfreq, const float* acc, bool* nothing) {
  if (nfreq < 1 || nfreq > mgbdft::kMaxFreq)
    return fail(MGB_ERR_ARGUMENT, "nfreq must be 1.." + std::to_string(mgbdft::kMaxFreq));
  if (nsamples < 0 || nsamples > mgbdft::kDepth)
    return fail(MGB_ERR_ARGUMENT, "nsamples must be 0.." + std::to_string(mgbdft::kDepth));
  if (ncols < 0 || ld < ncols) return fail(MGB_ERR_ARGUMENT, "ld must be at least ncols");
  if (samples == nullptr || omega == nullptr || acc == nullptr) return fail(MGB_ERR_ARGUMENT, "null argument");
  *nothing = (nsamples == 0 || ncols == 0);
  return MGB_OK;
}

int contract_with_table(const float* samples, int64_t ld, int64_t ncols, int32_t nsamples, const double* omega,
                        int32_t nfreq, int64_t first_step, int32_t step_stride, double dt, int32_t half_step_back,
                        double scale, float* acc, float* table, int* status, cudaStream_t s) {
  mgbdft::Contraction c = {};
  c.samples = samples;
  c.ld = ld;
  c.ncols = ncols;
  c.nsamples = nsamples;
  c.ncomp = 1;
  c.acc = acc;
  c.acc_ld = ncols;
  c.nfreq = nfreq;
  c.table = table;
  c.status = status;
  c.first_wait_ns = test_wait_limit(1);
  const cudaError_t err =
      mgbdft::launch_contraction(omega, first_step, step_stride, dt, half_step_back ? 1 : 0, scale, c, s);
  if (err != cudaSuccess) return cuda_error(err, "tensor-core DFT contraction");
  return MGB_OK;
}

}  // namespace

extern "C" {

size_t mgb_dft_scratch_bytes(int32_t nfreq) {
  if (nfreq < 1 || nfreq > mgbdft::kMaxFreq) return 0;
  return mgbdft::table_bytes(nfreq);
}

int mgb_dft_contract(const float* samples, int64_t ld, int64_t ncols, int32_t nsamples, const double* omega,
                     int32_t nfreq, int64_t first_step, int32_t step_stride, double dt, int32_t half_step_back,
                     double scale, float* acc, void* scratch, size_t scratch_bytes, void* stream) {
  bool nothing = false;
  const int rc = check_contract(samples, ld, ncols, nsamples, omega, nfreq, acc, &nothing);
  if (rc != MGB_OK) return rc;
  if (scratch == nullptr) return fail(MGB_ERR_ARGUMENT, "null argument");
  if (scratch_bytes < mgbdft::table_bytes(nfreq))
    return fail(MGB_ERR_ARGUMENT, "scratch is smaller than mgb_dft_scratch_bytes(nfreq)");
  if ((reinterpret_cast<uintptr_t>(scratch) & 15u) != 0) return fail(MGB_ERR_ARGUMENT, "scratch must be 16-byte aligned");
  if (nothing) return MGB_OK;
  StaticWords words;
  const int found = static_words(&words);
  if (found != MGB_OK) return found;
  return contract_with_table(samples, ld, ncols, nsamples, omega, nfreq, first_step, step_stride, dt,
                             half_step_back, scale, acc, static_cast<float*>(scratch), words.status,
                             static_cast<cudaStream_t>(stream));
}

// The phase table of this entry point is g_dft_table (the tile images of 2 *
// MGB_DFT_MAX_FREQ rows of MGB_DFT_DEPTH words, each word's two TF32 parts: 256 KB). No word of it must start at zero: the table kernel writes every
// word the contraction then reads. Calls that overlap on the device (different streams,
// or threads without ordering) share the one table and race.
int mgb_dft_contract_noalloc(const float* samples, int64_t ld, int64_t ncols, int32_t nsamples,
                             const double* omega, int32_t nfreq, int64_t first_step, int32_t step_stride,
                             double dt, int32_t half_step_back, double scale, float* acc, void* stream) {
  static_assert(sizeof(g_dft_table) >= mgbdft::kMaxTableBytes, "static table holds the largest contraction");
  // every refusal, and a call with no work, returns before the device is touched
  bool nothing = false;
  const int rc = check_contract(samples, ld, ncols, nsamples, omega, nfreq, acc, &nothing);
  if (rc != MGB_OK) return rc;
  if (nothing) return MGB_OK;
  StaticWords words;
  const int found = static_words(&words);
  if (found != MGB_OK) return found;
  return contract_with_table(samples, ld, ncols, nsamples, omega, nfreq, first_step, step_stride, dt,
                             half_step_back, scale, acc, static_cast<float*>(words.table), words.status,
                             static_cast<cudaStream_t>(stream));
}

int mgb_dft_contract_status(int32_t* dst, int32_t clear, void* stream) {
  if (dst == nullptr) return fail(MGB_ERR_ARGUMENT, "null argument");
  StaticWords words;
  const int found = static_words(&words);
  if (found != MGB_OK) return found;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t err = cudaMemcpyAsync(dst, words.status, sizeof(int32_t), cudaMemcpyDefault, s);
  if (err != cudaSuccess) return cuda_error(err, "contraction status read");
  if (clear != 0) {
    err = cudaMemsetAsync(words.status, 0, sizeof(int32_t), s);
    if (err != cudaSuccess) return cuda_error(err, "contraction status reset");
  }
  return MGB_OK;
}

}  // extern "C"

// ======================================================================================
// Field energy (the divergence guard's scalar)
//
// sum over the grid of |E|^2 eps + |B|^2 (eps = 1 / inverse permittivity of each E
// component; B is the H half's B word: the auxiliary's on its own-axis membership, H's
// elsewhere, where MEEP's H is B's word). Each cell's terms are formed in float32 and
// summed in float64 per thread, then per block, then into one device double.
namespace {

struct EnergyArgs {
  const float* E[3];
  const float* inv[3];
  const float* H[3];
  const float* B[3];  // NULL: no own-axis membership (H is B everywhere)
  int axis[3], a0[3], a1[3], b0[3], b1[3];
  int ny, nz;
  long long cells;
  double* out;
};

__global__ void __launch_bounds__(256) energy_kernel(const __grid_constant__ EnergyArgs a) {
  double sum = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long plane = (long long)a.ny * a.nz;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < a.cells; c += stride) {
    const int i = (int)(c / plane);
    const int rem = (int)(c - (long long)i * plane);
    const int at[3] = {i, rem / a.nz, rem % a.nz};
    float cell = 0.f;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const float e = a.E[q][c];
      cell += (e * e) / a.inv[q][c];
      float b = a.H[q][c];
      if (a.B[q] != nullptr) {
        const int r = at[a.axis[q]];
        if ((r >= a.a0[q] && r < a.a1[q]) || (r >= a.b0[q] && r < a.b1[q])) b = a.B[q][c];
      }
      cell += b * b;
    }
    sum += (double)cell;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, off);
  __shared__ double warp_sums[8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) warp_sums[warp] = sum;
  __syncthreads();
  if (warp == 0) {
    sum = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0.0;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, off);
    if (lane == 0) atomicAdd(a.out, sum);
  }
}

}  // namespace

extern "C" {

int mgb_field_energy(mgb_sim* sim, double* out, void* stream) {
  if (sim == nullptr || out == nullptr) return fail(MGB_ERR_ARGUMENT, "null argument");
  const mgb_sim_desc& d = sim->desc;
  EnergyArgs a = {};
  for (int q = 0; q < 3; ++q) {
    a.E[q] = d.E[q];
    a.inv[q] = d.inv_eps[q];
    a.H[q] = d.H[q];
    const mgb_aux& b = d.B[q];
    if (d.pml_active && b.data != nullptr && (b.a1 > b.a0 || b.b1 > b.b0)) {
      a.B[q] = b.data;
      a.axis[q] = b.axis;
      a.a0[q] = b.a0;
      a.a1[q] = b.a1;
      a.b0[q] = b.b0;
      a.b1[q] = b.b1;
    }
  }
  a.ny = d.ny;
  a.nz = d.nz;
  a.cells = (long long)d.nx * d.ny * d.nz;
  a.out = out;
  int device = 0, sms = 0;
  if (cudaGetDevice(&device) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return launch_error("device query");
  const long long blocks = std::min<long long>((long long)sms * 8, (a.cells + 255) / 256);
  energy_kernel<<<(unsigned)std::max<long long>(blocks, 1), 256, 0, static_cast<cudaStream_t>(stream)>>>(a);
  const cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return cuda_error(err, "field energy");
  return MGB_OK;
}

}  // extern "C"

// ======================================================================================
// Adjoint ABI
extern "C" {

int mgb_adjoint_step(mgb_sim* adj, const mgb_adjoint* a, int64_t step, void* stream) {
  if (adj == nullptr || a == nullptr || a->grad_inv == nullptr || a->d_after == nullptr)
    return fail(MGB_ERR_ARGUMENT, "null argument");
  if (adj->step.npoles != 0) return fail(MGB_ERR_UNSUPPORTED, "the adjoint step does not carry susceptibility poles");
  if (adj->has_cond) return fail(MGB_ERR_UNSUPPORTED, "the adjoint step does not carry a conductivity");
  if (adj->folded) return fail(MGB_ERR_UNSUPPORTED, "the adjoint step does not carry mirror folds");
  if (adj->step.inv) return fail(MGB_ERR_UNSUPPORTED, "the adjoint step is for 3-D runs");
  for (int q = 0; q < 3; ++q)
    if (a->mu_b[q] == nullptr || a->mu_d[q] == nullptr) return fail(MGB_ERR_ARGUMENT, "missing mu volume");
  const StepParams& p = adj->step;
  const int n[3] = {p.nx, p.ny, p.nz};
  for (int ax = 0; ax < 3; ++ax)
    if (a->box[2 * ax] < 0 || a->box[2 * ax] >= a->box[2 * ax + 1] || a->box[2 * ax + 1] > n[ax])
      return fail(MGB_ERR_ARGUMENT, "gradient box outside the grid");
  AdjParams ap;
  for (int q = 0; q < 3; ++q) {
    ap.mu_b[q] = a->mu_b[q];
    ap.mu_d[q] = a->mu_d[q];
  }
  for (int e = 0; e < 6; ++e) ap.box[e] = a->box[e];
  ap.d_after = a->d_after;
  ap.grad_inv = a->grad_inv;
  ap.first_step = step == 0 ? 1 : 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int xc = 4;
  const dim3 block(32, 4, 1);
  const dim3 grid((p.nz + 31) / 32, (p.ny + 3) / 4, (p.nx + xc - 1) / xc);
  const bool pml = adj->desc.pml_active != 0;
  if (pml) {
    adj_e<true><<<grid, block, 0, s>>>(p, ap, xc);
    adj_h<true><<<grid, block, 0, s>>>(p, ap, xc);
  } else {
    adj_e<false><<<grid, block, 0, s>>>(p, ap, xc);
    adj_h<false><<<grid, block, 0, s>>>(p, ap, xc);
  }
  return launch_error("adjoint step");
}

int mgb_adjoint_inject(mgb_sim* adj, int32_t monitor, int64_t post, void* stream) {
  if (adj == nullptr) return fail(MGB_ERR_ARGUMENT, "null plan");
  if (monitor < 0 || monitor >= adj->desc.nmonitors) return fail(MGB_ERR_ARGUMENT, "no such monitor");
  const StepParams& p = adj->step;
  const mgb_monitor& mon = adj->desc.monitors[monitor];
  DftParams q = {};
  q.nx = p.nx; q.ny = p.ny; q.nz = p.nz;
  for (int ax = 0; ax < 3; ++ax) q.met[ax] = p.met[ax];
  for (int c = 0; c < 3; ++c) { q.E[c] = p.E[c]; q.H[c] = p.H[c]; }
  q.mon = mon;
  const long long cells = (long long)(mon.region[1] - mon.region[0]) * (mon.region[3] - mon.region[2]) *
                          (mon.region[5] - mon.region[4]);
  const size_t smem = (size_t)mon.nfreq * 2 * sizeof(float2);
  adj_inject<<<(unsigned)((cells + 255) / 256), 256, smem, static_cast<cudaStream_t>(stream)>>>(q, post);
  return launch_error("adjoint injection");
}

int mgb_copy_box(mgb_sim* sim, int32_t family, const int32_t* box, float* dst, void* stream) {
  if (sim == nullptr || box == nullptr || dst == nullptr) return fail(MGB_ERR_ARGUMENT, "null argument");
  if (family < 0 || family > 2) return fail(MGB_ERR_ARGUMENT, "family is 0 (E), 1 (D) or 2 (H)");
  const StepParams& p = sim->step;
  const int n[3] = {p.nx, p.ny, p.nz};
  BoxArgs b;
  for (int ax = 0; ax < 3; ++ax) {
    if (box[2 * ax] < 0 || box[2 * ax] >= box[2 * ax + 1] || box[2 * ax + 1] > n[ax])
      return fail(MGB_ERR_ARGUMENT, "box outside the grid");
    b.box[2 * ax] = box[2 * ax];
    b.box[2 * ax + 1] = box[2 * ax + 1];
  }
  b.dst = dst;
  const long long cells = 3LL * (box[1] - box[0]) * (box[3] - box[2]) * (box[5] - box[4]);
  copy_box<<<(unsigned)((cells + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(p, family, b);
  return launch_error("box copy");
}

}  // extern "C"


// ======================================================================================
// Adjoint segment: one checkpoint interval recomputed and reversed in one call
extern "C" {

int mgb_adjoint_segment(mgb_sim* fwd, mgb_sim* adj, const mgb_adjoint* a, int64_t first_step, int32_t nsteps,
                        int32_t monitor, float* d_history, void* stream) {
  if (fwd == nullptr || adj == nullptr || a == nullptr || d_history == nullptr)
    return fail(MGB_ERR_ARGUMENT, "null argument");
  if (nsteps < 1) return fail(MGB_ERR_ARGUMENT, "a segment has at least one step");
  if (monitor < 0 || monitor >= adj->desc.nmonitors) return fail(MGB_ERR_ARGUMENT, "no such monitor");
  if (fwd->has_cond || adj->has_cond) return fail(MGB_ERR_UNSUPPORTED, "the adjoint step does not carry a conductivity");
  if (fwd->folded || adj->folded) return fail(MGB_ERR_UNSUPPORTED, "the adjoint step does not carry mirror folds");
  if (fwd->step.inv || adj->step.inv) return fail(MGB_ERR_UNSUPPORTED, "the adjoint step is for 3-D runs");
  int rc = check_words(fwd, first_step, nsteps);
  if (rc != MGB_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long box_cells =
      (long long)(a->box[1] - a->box[0]) * (a->box[3] - a->box[2]) * (a->box[5] - a->box[4]);
  // forward again from the restored checkpoint (the halves only: monitors are not
  // needed), keeping D over the box after every step
  for (int t = 0; t < nsteps; ++t) {
    const long long n = first_step + t;
    rc = launch_part(fwd, n, 0, s);
    if (rc == MGB_OK) rc = launch_part(fwd, n, 1, s);
    if (rc == MGB_OK) rc = mgb_copy_box(fwd, 1, a->box, d_history + (long long)t * 3 * box_cells, stream);
    if (rc != MGB_OK) return rc;
  }
  // then the adjoint back through the segment
  const int decimation = adj->desc.monitors[monitor].decimation;
  mgb_adjoint step_args = *a;
  for (int t = nsteps - 1; t >= 0; --t) {
    const long long n = first_step + t;
    if ((n + 1) % decimation == 0) {
      rc = mgb_adjoint_inject(adj, monitor, n + 1, stream);
      if (rc != MGB_OK) return rc;
    }
    step_args.d_after = d_history + (long long)t * 3 * box_cells;
    rc = mgb_adjoint_step(adj, &step_args, n, stream);
    if (rc != MGB_OK) return rc;
  }
  return launch_error("adjoint segment");
}

}  // extern "C"
