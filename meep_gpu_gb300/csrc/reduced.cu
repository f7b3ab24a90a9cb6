// The step kernels of reduced-dimension runs (2-D and 1-D: one periodic cell on each
// invariant axis). The per-cell arithmetic is the shared column marches of
// step_device.cuh compiled with RED, which drops a curl partner whose derivative lies
// along an invariant axis as MEEP's step plan does (fields.cpp figure_out_step_plan);
// the CTA-level dispatch is the generic kernels' (a march compiled for the PML axes the
// CTA reaches; a general march for CTAs at a Bloch face or holding magnetic sources).
#include "reduced.cuh"

namespace mgbred {

using namespace mgbstep;

namespace {

template <bool PML, bool COND, bool MSRC>
__global__ void __launch_bounds__(256, COND ? 4 : 5) h_reduced(const __grid_constant__ StepParams p,
                                                    const __grid_constant__ mgb_conductivity cp, int first_step,
                                                    int xchunk) {
  step_entry();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (k >= p.nz || j >= p.ny) return;
  const int i0 = (blockIdx.z + p.xbase) * xchunk, i1 = min(i0 + xchunk, p.nx);
  const mgb_conductivity* c = COND ? &cp : nullptr;
  if (cta_bloch(p, i0, blockIdx.y * blockDim.y, blockIdx.x * blockDim.x) ||
      (MSRC && cta_msrc(p, i0, i1, blockIdx.y * blockDim.y, blockDim.y, blockIdx.x * blockDim.x, blockDim.x))) {
    h_march<PML, COND, -1, true, true, true>(p, j, k, i0, i1, first_step, c);
    return;
  }
  if (!PML) {
    h_march<false, COND, -1, false, false, true>(p, j, k, i0, i1, first_step, c);
    return;
  }
#define MGB_MARCH(AXV, PMLV) h_march<PMLV, COND, AXV, false, false, true>(p, j, k, i0, i1, first_step, c)
  MGB_AXES_SWITCH(cta_axes(p, i0, i1, blockIdx.y * blockDim.y, blockDim.y, blockIdx.x * blockDim.x, blockDim.x),
                  MGB_MARCH)
#undef MGB_MARCH
}

template <bool PML, bool COND>
__global__ void __launch_bounds__(256, COND ? 4 : 5) e_reduced(const __grid_constant__ StepParams p,
                                                    const __grid_constant__ mgb_conductivity cp, int parity,
                                                    int xchunk) {
  step_entry();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (k >= p.nz || j >= p.ny) return;
  const int i0 = (blockIdx.z + p.xbase) * xchunk, i1 = min(i0 + xchunk, p.nx);
  const mgb_conductivity* c = COND ? &cp : nullptr;
  if (cta_bloch(p, i0, blockIdx.y * blockDim.y, blockIdx.x * blockDim.x)) {
    e_march<PML, COND, -1, true, true>(p, j, k, i0, i1, parity, p.src_words, c);
    return;
  }
  if (!PML) {
    e_march<false, COND, -1, false, true>(p, j, k, i0, i1, parity, p.src_words, c);
    return;
  }
#define MGB_MARCH(AXV, PMLV) e_march<PMLV, COND, AXV, false, true>(p, j, k, i0, i1, parity, p.src_words, c)
  MGB_AXES_SWITCH(cta_axes(p, i0, i1, blockIdx.y * blockDim.y, blockDim.y, blockIdx.x * blockDim.x, blockDim.x),
                  MGB_MARCH)
#undef MGB_MARCH
}

template <typename... KArgs, typename... Args>
cudaError_t launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, bool pdl, cudaStream_t s, Args&&... args) {
  if (!pdl) {
    kernel<<<grid, block, 0, s>>>(std::forward<Args>(args)...);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace

cudaError_t preload_kernels() {
  const void* kernels[] = {
      reinterpret_cast<const void*>(h_reduced<true, true, true>), reinterpret_cast<const void*>(h_reduced<true, true, false>),
      reinterpret_cast<const void*>(h_reduced<false, true, true>), reinterpret_cast<const void*>(h_reduced<false, true, false>),
      reinterpret_cast<const void*>(h_reduced<true, false, true>), reinterpret_cast<const void*>(h_reduced<true, false, false>),
      reinterpret_cast<const void*>(h_reduced<false, false, true>), reinterpret_cast<const void*>(h_reduced<false, false, false>),
      reinterpret_cast<const void*>(e_reduced<true, true>), reinterpret_cast<const void*>(e_reduced<false, true>),
      reinterpret_cast<const void*>(e_reduced<true, false>), reinterpret_cast<const void*>(e_reduced<false, false>)};
  for (const void* k : kernels) {
    cudaFuncAttributes attr;
    const cudaError_t err = cudaFuncGetAttributes(&attr, k);
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

cudaError_t launch_half(const StepParams& p, const mgb_conductivity& cp, bool cond, bool msrc, bool pml, int part,
                        int flag, dim3 grid, dim3 block, int xchunk, bool pdl, cudaStream_t s) {
  if (part == 0) {
    if (cond) {
      if (pml) return msrc ? launch(h_reduced<true, true, true>, grid, block, pdl, s, p, cp, flag, xchunk)
                           : launch(h_reduced<true, true, false>, grid, block, pdl, s, p, cp, flag, xchunk);
      return msrc ? launch(h_reduced<false, true, true>, grid, block, pdl, s, p, cp, flag, xchunk)
                  : launch(h_reduced<false, true, false>, grid, block, pdl, s, p, cp, flag, xchunk);
    }
    if (pml) return msrc ? launch(h_reduced<true, false, true>, grid, block, pdl, s, p, cp, flag, xchunk)
                         : launch(h_reduced<true, false, false>, grid, block, pdl, s, p, cp, flag, xchunk);
    return msrc ? launch(h_reduced<false, false, true>, grid, block, pdl, s, p, cp, flag, xchunk)
                : launch(h_reduced<false, false, false>, grid, block, pdl, s, p, cp, flag, xchunk);
  }
  if (cond) return pml ? launch(e_reduced<true, true>, grid, block, pdl, s, p, cp, flag, xchunk)
                       : launch(e_reduced<false, true>, grid, block, pdl, s, p, cp, flag, xchunk);
  return pml ? launch(e_reduced<true, false>, grid, block, pdl, s, p, cp, flag, xchunk)
             : launch(e_reduced<false, false>, grid, block, pdl, s, p, cp, flag, xchunk);
}

}  // namespace mgbred
