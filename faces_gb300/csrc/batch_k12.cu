// batch_k12.cu -- the batched kernel's form MODE = 1, H = 2 (batch_impl.cuh).
#include "batch_impl.cuh"

namespace faces {

cudaError_t batch_configure_12() { return batch_configure_t<1, 2>(); }

cudaError_t batch_launch_12(const BatchField *fields, const BatchUnit *units, int nunits, long grid, int run,
                            int nsmall, int wblocks, cudaStream_t s)
{
  return batch_launch_t<1, 2>(fields, units, nunits, grid, run, nsmall, wblocks, s);
}

}  // namespace faces
