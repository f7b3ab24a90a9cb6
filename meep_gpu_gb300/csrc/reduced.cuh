// Interface of the reduced-dimension step kernels (reduced.cu) to the library (meepgb.cu).
//
// A 2-D or 1-D run (StepParams::inv != 0: one periodic cell on each invariant axis) steps
// with kernels of its own, whatever the generic family its plan chose: every family
// computes the same words, and the marches these kernels run drop a curl partner whose
// derivative lies along an invariant axis (MEEP's step plan), which the 3-D kernels do
// not carry (the branch costs them registers). The launch shape and x chunk are the
// plan's.
#pragma once

#include "step_device.cuh"

namespace mgbred {

// One half (part 0 H, 1 E) of a reduced-dimension run over the chunks of `grid`;
// `flag` is the H half's first-step flag or the E half's parity; `cp` the conductivity
// (read only when `cond`). With `pdl` the launch is its stream predecessor's
// programmatic dependent (the kernels begin with step_entry).
cudaError_t launch_half(const mgbstep::StepParams& p, const mgb_conductivity& cp, bool cond, bool msrc, bool pml,
                        int part, int flag, dim3 grid, dim3 block, int xchunk, bool pdl, cudaStream_t s);

// Load every reduced-dimension kernel now (a plan's creation) rather than at its first
// launch: under lazy module loading that first launch fell inside a run's first timed
// call and cost it about 11 ms.
cudaError_t preload_kernels();

}  // namespace mgbred
