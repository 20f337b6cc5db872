// Matrix-free Schur PCG (filled in below).
#include "kernels.cuh"

namespace sfmba {

void launch_pcg_setup(const Bufs &, cudaStream_t) { throw Error(SFMBA_ERR_UNSUPPORTED, "PCG not built"); }
void launch_pcg_iteration(const Bufs &, cudaStream_t) { throw Error(SFMBA_ERR_UNSUPPORTED, "PCG not built"); }
void launch_pcg_finish(const Bufs &, cudaStream_t) { throw Error(SFMBA_ERR_UNSUPPORTED, "PCG not built"); }

}  // namespace sfmba
