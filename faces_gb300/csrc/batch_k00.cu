// batch_k00.cu -- the batched kernel's form MODE = 0, H = 0 (batch_impl.cuh).
#include "batch_impl.cuh"

namespace faces {

cudaError_t batch_configure_00() { return batch_configure_t<0, 0>(); }

cudaError_t batch_launch_00(const BatchField *fields, const BatchUnit *units, int nunits, long grid, int run,
                            int nsmall, int wblocks, cudaStream_t s)
{
  return batch_launch_t<0, 0>(fields, units, nunits, grid, run, nsmall, wblocks, s);
}

}  // namespace faces
