// The wavefront step kernel: a run of FDTD steps of one plan in one persistent launch
// (the item sequence and its dependencies are described in wave.cuh).
//
// This translation unit is compiled with every global load cached in L2 only
// (-Xptxas -dlcm=cg): within one launch a chunk's words are rewritten by other SMs, and an
// SM's L1 is not kept coherent with them. Read-only tables (coefficients, inverse
// permittivity, pole sigma) keep the read-only path. The per-cell arithmetic is the
// shared column marches of step_device.cuh, so every word equals the launch-per-half
// kernels' word.
#include "wave.cuh"

namespace mgbwave {

using namespace mgbstep;

namespace {

constexpr unsigned long long kWaitNs = 2000000000ull;  // ~2 s of wall time per dependency

__device__ __forceinline__ unsigned load_acquire(const unsigned* at) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(at) : "memory");
  return v;
}

// Publish one completed tile: a release reduction, so the tile's stores (every thread's,
// ordered before it by the CTA barrier) are visible to whoever reads the new count with
// acquire semantics.
__device__ __forceinline__ void add_release(unsigned* counter, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(counter), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait until *counter reaches target: true, or false when the wait ran out or another CTA
// gave up first (the abort flag), so no item ever waits past a failure.
__device__ bool wait_count(const unsigned* counter, unsigned target, const unsigned* abort_flag) {
  if (load_acquire(counter) >= target) return true;
  const unsigned long long start = now_ns();
  for (;;) {
    for (int spin = 0; spin < 32; ++spin) {
      if (load_acquire(counter) >= target) return true;
      __nanosleep(100);
    }
    if (load_acquire(abort_flag) != 0) return false;
    if (now_ns() - start > kWaitNs) return false;
  }
}

__device__ __forceinline__ unsigned* done_at(const WaveArgs& w, int t, int half, int c) {
  return w.done + ((long long)t * 2 + half) * w.chunks + c;
}

// A tile's columns of one half: the plain marches (PF false) or the prefetching ones
// (the next plane's loads issued ahead, z neighbours by shuffle), compiled for the axes
// whose memberships the tile reaches, as the launch-per-half kernels do.
template <bool PML, bool MSRC, bool PF>
__device__ __forceinline__ void h_tile_march(const StepParams& p, int j, int k, int i0, int i1, int j0, int by,
                                             int k0, int bz, int first_step) {
  if (MSRC && cta_msrc(p, i0, i1, j0, by, k0, bz)) {
    if (PF) h_march_pf<PML, -1, true>(p, j, k, i0, i1, first_step);
    else h_march<PML, false, -1, true>(p, j, k, i0, i1, first_step);
    return;
  }
  if (!PML) {
    if (PF) h_march_pf<false>(p, j, k, i0, i1, first_step);
    else h_march<false>(p, j, k, i0, i1, first_step);
    return;
  }
  if (PF) {
#define MGB_MARCH(AXV, PMLV) h_march_pf<PMLV, AXV>(p, j, k, i0, i1, first_step)
    MGB_AXES_SWITCH(cta_axes(p, i0, i1, j0, by, k0, bz), MGB_MARCH)
#undef MGB_MARCH
  } else {
#define MGB_MARCH(AXV, PMLV) h_march<PMLV, false, AXV>(p, j, k, i0, i1, first_step)
    MGB_AXES_SWITCH(cta_axes(p, i0, i1, j0, by, k0, bz), MGB_MARCH)
#undef MGB_MARCH
  }
}

template <bool PML, bool PF>
__device__ __forceinline__ void e_tile_march(const StepParams& p, int j, int k, int i0, int i1, int j0, int by,
                                             int k0, int bz, int parity, const double* words) {
  if (!PML) {
    if (PF) e_march_pf<false>(p, j, k, i0, i1, parity, words);
    else e_march<false>(p, j, k, i0, i1, parity, words);
    return;
  }
  if (PF) {
#define MGB_MARCH(AXV, PMLV) e_march_pf<PMLV, AXV>(p, j, k, i0, i1, parity, words)
    MGB_AXES_SWITCH(cta_axes(p, i0, i1, j0, by, k0, bz), MGB_MARCH)
#undef MGB_MARCH
  } else {
#define MGB_MARCH(AXV, PMLV) e_march<PMLV, false, AXV>(p, j, k, i0, i1, parity, words)
    MGB_AXES_SWITCH(cta_axes(p, i0, i1, j0, by, k0, bz), MGB_MARCH)
#undef MGB_MARCH
  }
}

template <bool PML, bool MSRC, bool PF>
__global__ void __launch_bounds__(256, PF ? 3 : 5) wave_step(const __grid_constant__ StepParams params,
                                                             const __grid_constant__ WaveArgs w) {
  // the parameters in shared memory: the source-word row changes with each item's step
  __shared__ StepParams sp;
  // the next item, taken while the current one is worked on (two slots, alternating, so
  // thread 0 never overwrites the one the other threads are still reading)
  __shared__ unsigned long long s_item[2];
  __shared__ int s_go;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int nthreads = blockDim.x * blockDim.y;
  {
    const int* src = reinterpret_cast<const int*>(&params);
    int* dst = reinterpret_cast<int*>(&sp);
    for (int at = tid; at < (int)(sizeof(StepParams) / sizeof(int)); at += nthreads) dst[at] = src[at];
  }
  const int bz = blockDim.x, by = blockDim.y;
  const int tiles = w.tiles_z * w.tiles_y;
  const unsigned long long per_block = (unsigned long long)w.window * 2 * w.chunks * tiles;
  unsigned long long* queue = reinterpret_cast<unsigned long long*>(w.control);
  const unsigned* abort_flag = w.control + 2;
  if (tid == 0) {
    // after a wait has run out anywhere, every CTA leaves at its next item
    s_item[0] = load_acquire(abort_flag) != 0 ? w.total : atomicAdd(queue, 1ull);
  }
  __syncthreads();
  for (int turn = 0;; turn ^= 1) {
    const unsigned long long v = s_item[turn];
    if (v >= w.total) return;
    const int block = (int)(v / per_block);
    const unsigned long long r = v - (unsigned long long)block * per_block;
    const int entry = (int)(r / tiles);
    const int tile = (int)(r - (unsigned long long)entry * tiles);
    const unsigned code = w.table[entry];
    const int k_step = (int)(code >> 20), half = (int)((code >> 16) & 15u), c = (int)(code & 0xffffu);
    const int t = block * w.window + k_step;
    const bool live = t < w.steps;  // uniform over the CTA
    const long long n = w.first + t;
    if (tid == 0) {
      bool ok = live && load_acquire(abort_flag) == 0;
      if (ok && half == 0) {
        if (t > 0) {
          ok = wait_count(done_at(w, t - 1, 1, c), tiles, abort_flag);
          if (ok && c + 1 < w.chunks) ok = wait_count(done_at(w, t - 1, 1, c + 1), tiles, abort_flag);
        }
      } else if (ok) {
        ok = wait_count(done_at(w, t, 0, c), tiles, abort_flag);
        if (ok && c > 0) ok = wait_count(done_at(w, t, 0, c - 1), tiles, abort_flag);
      }
      if (live && !ok) {
        if (sp.status != nullptr) atomicOr(sp.status, 8);
        atomicExch(w.control + 2, 1u);
      }
      s_go = ok ? 1 : 0;
      sp.src_words = (sp.nsrc > 0 && live) ? w.words + (n - w.words_first) * sp.nsrc : nullptr;
      // the next item, while this one is worked on: its dependencies are earlier items,
      // this one's among them at most, which this CTA finishes first
      s_item[turn ^ 1] = load_acquire(abort_flag) != 0 ? w.total : atomicAdd(queue, 1ull);
    }
    __syncthreads();
    if (s_go) {
      const int tz = tile % w.tiles_z, ty = tile / w.tiles_z;
      const int k0 = tz * bz, j0 = ty * by;
      const int k = k0 + threadIdx.x, j = j0 + threadIdx.y;
      const int i0 = c * w.xchunk, i1 = min(i0 + w.xchunk, sp.nx);
      if (k < sp.nz && j < sp.ny) {
        if (half == 0)
          h_tile_march<PML, MSRC, PF>(sp, j, k, i0, i1, j0, by, k0, bz, (int)(n == 0));
        else
          e_tile_march<PML, PF>(sp, j, k, i0, i1, j0, by, k0, bz, (int)(n & 1), sp.src_words);
      }
    }
    __syncthreads();  // every thread's stores of the item are issued; sp is free again
    if (tid == 0 && live) add_release(done_at(w, t, half, c), 1u);
  }
}

// One block's chunk items in sequence order (one thread: a few thousand entries). At
// position pos, for each step k of the block: the H half of chunk pos - skew k, then the
// E half of chunk pos - skew k - 1, so every item's dependencies lie at least one whole
// position earlier in the sequence.
__global__ void wave_table(unsigned* table, int window, int chunks) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  int at = 0;
  const int positions = chunks + 1 + kSkew * (window - 1);
  for (int pos = 0; pos < positions; ++pos) {
    for (int k = 0; k < window; ++k) {
      const int ch = pos - kSkew * k;
      if (ch >= 0 && ch < chunks) table[at++] = ((unsigned)k << 20) | (0u << 16) | (unsigned)ch;
      const int ce = ch - 1;
      if (ce >= 0 && ce < chunks) table[at++] = ((unsigned)k << 20) | (1u << 16) | (unsigned)ce;
    }
  }
}

template <bool PML, bool MSRC, bool PF>
const void* wave_kernel() {
  return reinterpret_cast<const void*>(wave_step<PML, MSRC, PF>);
}

template <bool PF>
void launch_family(const StepParams& p, const WaveArgs& w, int blocks, dim3 block, bool pml, bool msrc,
                   cudaStream_t s) {
  if (pml && msrc) wave_step<true, true, PF><<<blocks, block, 0, s>>>(p, w);
  else if (pml) wave_step<true, false, PF><<<blocks, block, 0, s>>>(p, w);
  else if (msrc) wave_step<false, true, PF><<<blocks, block, 0, s>>>(p, w);
  else wave_step<false, false, PF><<<blocks, block, 0, s>>>(p, w);
}

}  // namespace

cudaError_t launch_wave(const StepParams& p, const WaveArgs& w, int blocks, dim3 block, int family, bool pml,
                        bool msrc, cudaStream_t s) {
  if (family == 2) launch_family<true>(p, w, blocks, block, pml, msrc, s);
  else launch_family<false>(p, w, blocks, block, pml, msrc, s);
  return cudaGetLastError();
}

cudaError_t launch_wave_table(unsigned* table, int window, int chunks, cudaStream_t s) {
  wave_table<<<1, 32, 0, s>>>(table, window, chunks);
  return cudaGetLastError();
}

int wave_blocks_per_sm(int threads, int family, bool pml, bool msrc) {
  const bool pf = family == 2;
  const void* fn = pf ? (pml ? (msrc ? wave_kernel<true, true, true>() : wave_kernel<true, false, true>())
                             : (msrc ? wave_kernel<false, true, true>() : wave_kernel<false, false, true>()))
                      : (pml ? (msrc ? wave_kernel<true, true, false>() : wave_kernel<true, false, false>())
                             : (msrc ? wave_kernel<false, true, false>() : wave_kernel<false, false, false>()));
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, threads, 0) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return blocks;
}

}  // namespace mgbwave
