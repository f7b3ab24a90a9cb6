// Interface of the wavefront step kernel (wave.cu) to the library (meepgb.cu).
//
// A run of steps of one plan in one persistent launch. The work is a sequence of items
// (step t, half, x chunk c, (y, z) tile) that resident CTAs take in order from a global
// counter. The sequence is cut into blocks of `window` steps; within a block it sweeps the
// chunks by position, and at position pos it holds, for k = 0 .. window - 1, every tile of
// the H half of step k at chunk pos - skew * k and then of its E half one chunk behind.
// So a chunk is visited by the block's steps one after the other while its neighbourhood
// is still in L2, and each word is brought from HBM about once per window instead of
// once per step; every dependency of an item lies at least one position earlier, which
// leaves the CTAs a position's worth of items to work on while it completes.
//
// Dependencies are per chunk, on completion counters (tiles done) that an item waits on
// before it starts (bounded; see wave.cu): H(t, c) after E(t-1, c) and E(t-1, c+1) (the
// curl reads E one plane above; H(t, c) also overwrites the H that E(t-1, c+1) read), and
// E(t, c) after H(t, c) and H(t, c-1) (the curl reads H one plane below; H(t, c-1) read
// this chunk's E). Every item waits only on items earlier in the sequence, which CTAs took
// before it and which wait on nothing later, so the launch always completes. The x axis
// must be metallic (a periodic x would make chunk 0 wait on the last chunk).
#pragma once

#include "step_device.cuh"

namespace mgbwave {

constexpr int kMaxWindow = 16;
constexpr int kSkew = 3;
constexpr int kControlWords = 64;  // queue counter, abort flag (256 bytes)

struct WaveArgs {
  unsigned* control;        // [0..1] the 64-bit item counter, [2] the abort flag
  const unsigned* table;    // one block's chunk items: (k << 20) | (half << 16) | chunk
  unsigned* done;           // [steps][2][chunks] tiles completed
  const double* words;      // source deposit words [steps][nsrc] from step words_first
  long long words_first;
  long long first;          // the run's first step
  int steps;                // steps in the run
  int window;               // steps per block
  int chunks;               // x chunks
  int xchunk;               // planes per chunk
  int tiles_z, tiles_y;     // (y, z) tiles per chunk
  unsigned long long total; // items of the run's blocks (a block's items past the run are skipped)
};

// Entries of one block's table: window * 2 * chunks.
inline int table_entries(int window, int chunks) { return window * 2 * chunks; }

// family 0: the plain column marches; 2: the prefetching ones.
cudaError_t launch_wave(const mgbstep::StepParams& p, const WaveArgs& w, int blocks, dim3 block, int family,
                        bool pml, bool msrc, cudaStream_t s);
cudaError_t launch_wave_table(unsigned* table, int window, int chunks, cudaStream_t s);
// Resident CTAs of `threads` threads per SM for the kernel variant (0 on error).
int wave_blocks_per_sm(int threads, int family, bool pml, bool msrc);

}  // namespace mgbwave
