// Tensor-core DFT contraction: acc[2 nfreq x N] += P[2 nfreq x K] . S[K x N] per
// component, on the tcgen05 tensor cores (kind::tf32, accumulator in tensor memory),
// with the 3xTF32 split for float32 accuracy. See dft_tc.cuh for the interface.
//
// Reference counterpart: the per-step accumulation of DFTMonitor.update /
// FluxMonitor.update (meep_gpu/dft.py:2197, :3031), which adds phase * sample into every
// accumulator word at each decimated step; here K such steps are buffered and added in
// one pass, so the accumulators are read and written once per K samples.
//
// The table kernel writes the phase rows already split into TF32 high and low parts, in
// the shared-memory image the MMAs read (canonical K-major layout without swizzle), one
// 32 KB image per 128-row tile. One CTA (eight warps) owns a 128-column tile of one
// component: it loads its samples (K = 32 rows), asks L2 for the accumulator rows it
// will add to, stages the samples in shared memory as TF32 high and low parts, then for
// each 128-row tile of phases copies the tile's image into shared memory with one bulk
// asynchronous copy (cp.async.bulk, completing on an mbarrier), one thread issues the 12
// MMAs (4 K-slices x 3 products) into a 128 x 128 float32 accumulator in tensor memory,
// and every warp reads its 32 lanes back (tcgen05.ld) and adds them to the accumulators
// in global memory through a shared-memory transpose (coalesced rows).
#include "dft_tc.cuh"

#include <cstdint>

namespace mgbdft {
namespace {

constexpr int kRows = 128;           // M per tile = tensor-memory lanes
constexpr int kCols = 128;           // N per tile = tensor-memory columns (3 CTAs per SM)
constexpr int kThreads = 256;        // warp w reads lanes 32(w % 4) .. + 31, columns half w / 4
constexpr int kSlices = kDepth / 8;  // kind::tf32 takes K = 8 per MMA
// K-major without swizzle: core matrices of 8 rows x 16 bytes (4 elements). In one K
// slice (8 elements, 32 bytes a row) the two core matrices of a row group are 128 bytes
// apart (leading byte offset) and consecutive 8-row groups 256 bytes apart (stride
// byte offset); slice j of a tile starts j * rows * 32 bytes in.
constexpr unsigned kLBO = 128;
constexpr unsigned kSBO = 256;
constexpr int kSliceA = kRows * 32;
constexpr int kSliceB = kCols * 32;
constexpr int kTileA = kSliceA * kSlices;  // 16 KB
constexpr int kTileB = kSliceB * kSlices;  // 32 KB
constexpr int kSmemBytes = 2 * kTileB + 2 * kTileA + 64;
constexpr int kTableTile = 2 * kTileA;  // bytes of one 128-row tile's phase image (high, low)
// Instruction descriptor: D float32 (bits 4-5 = 1), A and B TF32 (bits 7-9, 10-12 = 2),
// both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr unsigned kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((unsigned)(kCols >> 3) << 17) |
                            ((unsigned)(kRows >> 4) << 24);
static_assert(kDepth % 8 == 0, "K slices of 8");
static_assert(kSmemBytes <= 227 * 1024, "shared memory");
static_assert((kThreads / 32) * 32 * 17 * 4 <= 2 * kTileA, "epilogue staging fits in the phase tiles");

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ int kmajor_offset(int r, int k, int slice_bytes) {
  return (k >> 3) * slice_bytes + (r >> 3) * (int)kSBO + ((k >> 2) & 1) * (int)kLBO + (r & 7) * 16 +
         (k & 3) * 4;
}

// Shared-memory matrix descriptor: start address, leading and stride byte offsets (each
// >> 4), descriptor version 1 at bit 46, no swizzle.
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr) {
  return (unsigned long long)((addr >> 4) & 0x3FFFu) |
         ((unsigned long long)((kLBO >> 4) & 0x3FFFu) << 16) |
         ((unsigned long long)((kSBO >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ float to_tf32(float x) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void tmem_alloc(unsigned* slot, unsigned ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(unsigned taddr, unsigned ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void mma_tf32(unsigned tmem_d, unsigned long long a, unsigned long long b,
                                         unsigned accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(unsigned long long* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(unsigned taddr, unsigned (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Arm the barrier's phase for `bytes` of asynchronous copies (this thread's arrival).
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// One bulk copy global -> shared (both 16-byte aligned, bytes a multiple of 16), counted
// on the barrier's transaction bytes.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

constexpr unsigned long long kWaitLimitNs = 1000000000ull;  // ~1 s of wall time

// Wait for phase `parity` of the MMA barrier for at most limit_ns of wall time; a limit
// of 0 gives up without looking (the test hook that makes a wait run out).
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  unsigned long long limit_ns = kWaitLimitNs) {
  if (limit_ns == 0) return false;
  if (mbar_try_wait(bar, parity)) return true;
  unsigned long long start, now;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(start));
  for (;;) {
    for (int spin = 0; spin < 256; ++spin)
      if (mbar_try_wait(bar, parity)) return true;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
    if (now - start > limit_ns) return false;
  }
}

__device__ __forceinline__ int rows_of(int nfreq) { return ((2 * nfreq + kRows - 1) / kRows) * kRows; }

// Row m, sample k of the phase table as its tile's shared-memory image: the TF32 high
// part at the K-major offset of (m mod 128, k) in the tile's first 16 KB, the low part
// (the TF32 rounding of what the high part leaves) at the same offset in the second.
__device__ __forceinline__ void put_phase(float* table, int m, int k, float v) {
  const float h = to_tf32(v);
  const float l = to_tf32(v - h);
  unsigned char* tile = reinterpret_cast<unsigned char*>(table) + (size_t)(m / kRows) * kTableTile;
  const int off = kmajor_offset(m % kRows, k, kSliceA);
  *reinterpret_cast<float*>(tile + off) = h;
  *reinterpret_cast<float*>(tile + kTileA + off) = l;
}

// One thread per (frequency, sample): the cosine and sine rows of one angle (rows 2f and
// 2f + 1), zero in the padding rows and past nsamples.
__global__ void __launch_bounds__(64) table_kernel(const double* __restrict__ omega, int nfreq,
                                                   long long first_post, int stride, double dt,
                                                   int half_back, double scale, int nsamples,
                                                   float* __restrict__ table) {
  // the contraction that follows may start now: it reads this table only after
  // griddepcontrol.wait, which waits for this grid to complete
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  const int pairs = rows_of(nfreq) / 2;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= pairs * kDepth) return;
  const int f = idx / kDepth, k = idx % kDepth;
  float vc = 0.f, vs = 0.f;
  if (f < nfreq && k < nsamples) {
    // the same float64 expressions as the step-by-step phases
    const long long post = first_post + (long long)k * stride;
    const double t_e = (double)post * dt;
    const double t = half_back ? t_e - 0.5 * dt : t_e;
    double s, co;
    sincos(t * omega[f], &s, &co);
    vc = (float)(co * scale);
    vs = (float)(s * scale);
  }
  put_phase(table, 2 * f, k, vc);
  put_phase(table, 2 * f + 1, k, vs);
}

__global__ void __launch_bounds__(kThreads, 3) contract_kernel(const __grid_constant__ Contraction c) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* b_hi = smem;
  unsigned char* b_lo = smem + kTileB;
  unsigned char* a_hi = smem + 2 * kTileB;
  unsigned char* a_lo = a_hi + kTileA;
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(a_lo + kTileA);  // MMA commits
  unsigned long long* tbar = bar + 1;                                               // phase copies
  unsigned* tmem_slot = reinterpret_cast<unsigned*>(bar + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int q = blockIdx.y;
  static_assert(kThreads == 256, "two warps per 32 tensor-memory lanes");
  const long long n0 = (long long)blockIdx.x * kCols;

  const int mpad = rows_of(c.nfreq);
  const int mrows = 2 * c.nfreq;
  float* acc = c.acc + c.acc_off[q];
  // Samples: rows k < nsamples of this component's columns [n0, n0 + 128), zero beyond,
  // loaded first (all in flight together): the staging waits for them.
  const float* src = c.samples + c.sample_off[q];
  constexpr int kPerThread = kDepth * kCols / kThreads;
  float v[kPerThread];
#pragma unroll
  for (int u = 0; u < kPerThread; ++u) {
    const int idx = tid + u * kThreads;
    const int k = idx / kCols, n = idx % kCols;
    v[u] = (k < c.nsamples && n0 + n < c.ncols) ? __ldcs(src + (long long)k * c.ld + n0 + n) : 0.f;
  }
  // Then the accumulator rows of this tile (2 nfreq rows of 128 columns, 512 bytes each)
  // requested into L2: their DRAM reads overlap the staging and the MMAs instead of
  // waiting in the epilogue. (The memory clobber keeps the sample loads issued first.)
  for (int at = tid; at < mrows * (kCols / 32); at += kThreads) {
    const int r = at / (kCols / 32);
    const long long n = n0 + (at % (kCols / 32)) * 32;
    if (n < c.ncols)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(acc + (long long)r * c.acc_ld + n) : "memory");
  }
  if (warp == 0) tmem_alloc(tmem_slot, kCols);
  const int tiles = mpad / kRows;
  const unsigned char* table = reinterpret_cast<const unsigned char*>(c.table);
  if (tid == 0) {
    mbar_init(bar);
    mbar_init(tbar);
    // the first phase tile's image, in flight while the samples are staged, once the
    // table kernel this launch depends on has completed (everything else this kernel
    // reads was written before that kernel began)
    asm volatile("griddepcontrol.wait;" ::: "memory");
    mbar_expect_tx(tbar, kTableTile);
    bulk_load(a_hi, table, kTableTile, tbar);
  }
#pragma unroll
  for (int u = 0; u < kPerThread; ++u) {
    const int idx = tid + u * kThreads;
    const int k = idx / kCols, n = idx % kCols;
    const float h = to_tf32(v[u]);
    const float l = to_tf32(v[u] - h);
    const int off = kmajor_offset(n, k, kSliceB);
    *reinterpret_cast<float*>(b_hi + off) = h;
    *reinterpret_cast<float*>(b_lo + off) = l;
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const unsigned tmem = *tmem_slot;
  unsigned parity = 0, tparity = 0;
  for (int mt = 0; mt < tiles; ++mt) {
    // thread 0: the tile's phase image has landed (bounded wait), then the MMAs
    bool landed = true;
    if (tid == 0) {
      landed = mbar_wait_bounded(tbar, tparity);
      if (landed) {
#pragma unroll
        for (int j = 0; j < kSlices; ++j) {
          const unsigned long long ah = smem_desc(smem_u32(a_hi + j * kSliceA));
          const unsigned long long al = smem_desc(smem_u32(a_lo + j * kSliceA));
          const unsigned long long bh = smem_desc(smem_u32(b_hi + j * kSliceB));
          const unsigned long long bl = smem_desc(smem_u32(b_lo + j * kSliceB));
          mma_tf32(tmem, ah, bh, j > 0 ? 1u : 0u);
          mma_tf32(tmem, ah, bl, 1u);
          mma_tf32(tmem, al, bh, 1u);
        }
        mma_commit(bar);
      }
    }
    if (__syncthreads_or(!landed)) {
      // The copy did not land in time: report, give it one more wait with the normal
      // bound (shared memory is released only once it has landed, or that wait has run
      // out too), and leave without an MMA.
      if (tid == 0) {
        if (c.status != nullptr) atomicOr(c.status, 4);
        mbar_wait_bounded(tbar, tparity);
      }
      __syncthreads();
      break;
    }
    tparity ^= 1u;
    const unsigned long long limit =
        (mt == 0 && c.first_wait_ns >= 0) ? (unsigned long long)c.first_wait_ns : kWaitLimitNs;
    bool ok = mbar_wait_bounded(bar, parity, limit);
    ok = __syncthreads_and(ok) != 0;
    if (!ok) {
      // The MMAs did not complete in time: report, give them one more wait with the
      // normal bound (tensor memory is freed only once they have completed, or that wait
      // has run out too), and leave without touching the accumulators.
      if (tid == 0 && c.status != nullptr) atomicOr(c.status, 4);
      mbar_wait_bounded(bar, parity);
      __syncthreads();
      break;
    }
    parity ^= 1u;
    fence_after_sync();
    // Epilogue: warp w reads its 32 lanes (rows) of one half of the columns 16 at a
    // time, turns them round in shared memory (the phase tile's space, free once the
    // MMAs are done; rows padded to 17 words, so neither side conflicts), and adds them
    // to the accumulators with each half-warp on 16 consecutive columns of a row.
    const int lane_base = (warp & 3) * 32;
    const int c_begin = (warp >> 2) * (kCols / 2);
    float* stage = reinterpret_cast<float*>(a_hi) + warp * (32 * 17);
    const int col = lane & 15, rh = (lane >> 4) * 16;
#pragma unroll 1
    for (int c0 = c_begin; c0 < c_begin + kCols / 2; c0 += 16) {
      unsigned v[16];
      tmem_ld16(tmem + ((unsigned)lane_base << 16) + (unsigned)c0, v);
#pragma unroll
      for (int j = 0; j < 16; ++j) stage[lane * 17 + j] = __uint_as_float(v[j]);
      __syncwarp();
      const long long n = n0 + c0 + col;
      if (n < c.ncols) {
        // all 16 reads first (in flight together), then the adds and writes
        float old[16];
        const int m0 = mt * kRows + lane_base + rh;
        float* a0 = acc + (long long)m0 * c.acc_ld + n;
#pragma unroll
        for (int r = 0; r < 16; ++r) old[r] = (m0 + r < mrows) ? a0[(long long)r * c.acc_ld] : 0.f;
#pragma unroll
        for (int r = 0; r < 16; ++r)
          if (m0 + r < mrows) a0[(long long)r * c.acc_ld] = old[r] + stage[(rh + r) * 17 + col];
      }
      __syncwarp();
    }
    // the staging's generic-proxy accesses ordered before the next image's bulk copy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    fence_before_sync();
    __syncthreads();  // tensor memory and the phase tile are free for the next tile
    if (tid == 0 && mt + 1 < tiles) {
      mbar_expect_tx(tbar, kTableTile);
      bulk_load(a_hi, table + (size_t)(mt + 1) * kTableTile, kTableTile, tbar);
    }
  }
  fence_after_sync();
  if (warp == 0) tmem_dealloc(tmem, kCols);
}

}  // namespace

int table_rows(int nfreq) { return ((2 * nfreq + kRows - 1) / kRows) * kRows; }

size_t table_bytes(int nfreq) { return (size_t)(table_rows(nfreq) / kRows) * kTableTile; }

cudaError_t preload_kernels() {
  cudaFuncAttributes attr;
  cudaError_t err = cudaFuncGetAttributes(&attr, reinterpret_cast<const void*>(table_kernel));
  if (err == cudaSuccess) err = cudaFuncGetAttributes(&attr, reinterpret_cast<const void*>(contract_kernel));
  return err;
}

cudaError_t launch_contraction(const double* omega, long long first_post, int stride, double dt, int half_back,
                               double scale, const Contraction& c, cudaStream_t stream) {
  static_assert(kTableTile == kRows * kDepth * 2 * sizeof(float), "a tile image holds its rows' two parts");
  static_assert(kMaxTableBytes == (size_t)(2 * kMaxFreq / kRows) * kTableTile, "the largest table");
  // the bulk copies of the phase images start 16-byte aligned
  if ((reinterpret_cast<uintptr_t>(c.table) & 15u) != 0) return cudaErrorInvalidValue;
  if (c.ncols <= 0 || c.ncomp <= 0) return cudaSuccess;
  // per device, so set at every launch (contractions are rare: one per kDepth samples)
  cudaError_t err = cudaFuncSetAttribute(contract_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
  if (err != cudaSuccess) return err;
  // the table: one (cosine, sine) pair a thread, in blocks of 64 so the float64 work
  // spreads over many SMs
  const int total = table_rows(c.nfreq) / 2 * kDepth;
  table_kernel<<<(total + 63) / 64, 64, 0, stream>>>(omega, c.nfreq, first_post, stride, dt, half_back, scale,
                                                     c.nsamples, const_cast<float*>(c.table));
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  // the contraction as the table kernel's programmatic dependent: its CTAs start while
  // the table is formed, load their samples and request their accumulators, and wait
  // for the table grid (griddepcontrol.wait) only before the first phase copy
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)((c.ncols + kCols - 1) / kCols), (unsigned)c.ncomp, 1);
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = kSmemBytes;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, contract_kernel, c);
}

}  // namespace mgbdft
