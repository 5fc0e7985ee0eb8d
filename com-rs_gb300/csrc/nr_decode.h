// Host interface of the graph-specialised f32 layered decoder (layered_nr.cuh,
// decode_nr.cu), called by the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "code_host.h"
#include "layered_nr.cuh"

namespace cbk {

// A decoder kernel for one code: the base graph's nvcc-built kernel (Z and shifts from
// the launch parameters), or the code's own, compiled at run time with Z and the shifts
// as constants.
struct NrKernel {
  const void* fn = nullptr;  // launchable handle (a __global__ function or a cudaKernel_t)
  bool specialized = false;
  bool library = false;      // fn is a cudaKernel_t of a run-time compiled library
};

// the code part and tables of the launch parameters
void fill_nr_args(const cbh::NrCode& h, cbn::NrArgs& a);

// The kernel for `h` on `device`: its own specialisation when `specialize` is set and the
// run-time compiler is at hand (built once per base graph and lifting size, then taken
// from the process's cache or the on-disk cache), else the base graph's kernel.  `note`
// receives why no specialisation is used, if none is.  `learned`: the learned min-sum's
// kernel (layered_nr_kernel with NrLearnedArgs) instead of the plain decoder's; `rule` the
// plain decoder's min-sum rule (cbd::RULE_NMS or RULE_OMS), compiled into its
// specialisation.
NrKernel nr_kernel(const cbh::NrCode& h, int device, bool specialize, std::string* note, bool learned = false,
                   int rule = 1);

// resident CTAs of the persistent grid (occupancy x SMs) and the launch
int nr_grid_size(const NrKernel& k, const cbh::NrCode& h, int device);
size_t nr_smem(const cbh::NrCode& h);
cudaError_t nr_launch(const NrKernel& k, const cbn::NrArgs& a, int grid, cudaStream_t stream);
int nr_learned_grid_size(const NrKernel& k, const cbh::NrCode& h, int device);
cudaError_t nr_learned_launch(const NrKernel& k, const cbn::NrLearnedArgs& la, int grid, cudaStream_t stream);

// Compile (without a GPU) and store in the on-disk cache the specialisation of `h`;
// returns false with the reason in `note` when the run-time compiler is missing or fails.
bool nr_prepare(const cbh::NrCode& h, std::string* note, bool learned = false, int rule = 1);

}  // namespace cbk
