// batch_k20.cu -- the batched kernel's form MODE = 2, H = 0 (batch_impl.cuh).
#include "batch_impl.cuh"

namespace faces {

cudaError_t batch_configure_20() { return batch_configure_t<2, 0>(); }

cudaError_t batch_launch_20(const BatchField *fields, const BatchUnit *units, int nunits, long grid, int run,
                            int nsmall, int wblocks, cudaStream_t s)
{
  return batch_launch_t<2, 0>(fields, units, nunits, grid, run, nsmall, wblocks, s);
}

}  // namespace faces
