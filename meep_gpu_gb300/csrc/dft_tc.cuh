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
  const float* table;                   // [mpad][kDepth] phase rows (see launch_table)
  int* status;                          // ORed with 4 when a tensor-core wait times out
  long long first_wait_ns;              // limit of the first tile's wait; negative: the normal
                                        // limit (a test hook: 0 gives up before waiting)
};

// Rows of the phase table: 2 * nfreq rounded up to the 128-row tile.
int table_rows(int nfreq);
// Bytes of the phase table for nfreq frequencies.
size_t table_bytes(int nfreq);

// Phase rows for samples taken after steps first_post + k * stride (k < nsamples) at
// t = post * dt, less dt / 2 when half_back; rows 2f, 2f + 1 = cos, sin times scale;
// every other entry of the [table_rows][kDepth] table is written as zero.
cudaError_t launch_table(const double* omega, int nfreq, long long first_post, int stride,
                         double dt, int half_back, double scale, int nsamples, float* table,
                         cudaStream_t stream);

// acc += P . S for every component of the contraction (one launch).
cudaError_t launch_contract(const Contraction& c, cudaStream_t stream);

}  // namespace mgbdft
