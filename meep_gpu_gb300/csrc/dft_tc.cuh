// Internal interface of the tensor-core DFT contraction (dft_tc.cu).
//
// A DFT monitor buffers the cell-centred samples of up to kDepth accumulation steps,
// then adds them to its accumulators in one contraction per component:
//   acc[2f + 0][n] += sum_k cos(w_f t_k) * scale * sample[k][n]
//   acc[2f + 1][n] += sum_k sin(w_f t_k) * scale * sample[k][n]
// i.e. acc[M x N] += P[M x K] . S[K x N], M = 2 * nfreq, on the tcgen05 tensor cores in
// TF32 with the 3xTF32 split (P = Ph + Pl, S = Sh + Sl, P.S ~ Ph.Sh + Ph.Sl + Pl.Sh),
// which keeps float32 accuracy. The phases are formed in float64 on the device exactly
// as the step-by-step accumulation forms them (t = post * dt, minus dt/2 for H).
#pragma once

#include <cuda_runtime.h>

namespace mgbdft {

constexpr int kDepth = 32;     // samples per contraction (K)
constexpr int kMaxFreq = 512;  // 2 * kMaxFreq phase rows at most
constexpr int kMaxComps = 6;
// Bytes of the largest phase table: 2 * kMaxFreq rows (a multiple of the 128-row tile),
// each word as its TF32 high and low parts.
constexpr size_t kMaxTableBytes = (size_t)2 * kMaxFreq * kDepth * 2 * sizeof(float);

struct Contraction {
  const float* samples;                 // rows k < kDepth, row stride ld
  long long ld;
  long long ncols;                      // columns of each component
  int nsamples;                         // rows in use; rows beyond read as zero
  int ncomp;                            // components contracted by this launch
  long long sample_off[kMaxComps];      // first column of component q
  float* acc;                           // component q: acc + acc_off[q], [2 nfreq][acc_ld]
  long long acc_off[kMaxComps];
  long long acc_ld;
  int nfreq;
  const float* table;                   // phase tiles' shared-memory images (launch_contraction),
                                        // 16-byte aligned
  int* status;                          // ORed with 4 when a tensor-core wait times out
  long long first_wait_ns;              // limit of the first tile's wait; negative: the normal
                                        // limit (a test hook: 0 gives up before waiting)
};

// Rows of the phase table: 2 * nfreq rounded up to the 128-row tile.
int table_rows(int nfreq);
// Bytes of the phase table for nfreq frequencies.
size_t table_bytes(int nfreq);

// One contraction: the phase table into c.table, then acc += P . S for every component
// of c (one launch each). Phase rows for samples taken after steps first_post + k *
// stride (k < c.nsamples) at t = post * dt, less dt / 2 when half_back; rows 2f, 2f + 1 =
// cos, sin times scale; every other entry of the table_rows x kDepth phases is zero. The
// table is written as each 128-row tile's shared-memory image for the MMAs: the TF32
// high parts in the canonical K-major layout (16 KB), then the low parts (16 KB). The
// contraction kernel is launched as the table kernel's programmatic dependent.
cudaError_t launch_contraction(const double* omega, long long first_post, int stride, double dt,
                               int half_back, double scale, const Contraction& c, cudaStream_t stream);

// Load the table and contraction kernels now (a plan's creation) rather than at a run's
// first flush, which under lazy module loading can fall inside its timed steps.
cudaError_t preload_kernels();

}  // namespace mgbdft
