// chain_f32_g1.cu -- one instantiation of the chain kernel (F32 = true, GN = 1).
#include "chain_kernel.cuh"

namespace fmc {
template cudaError_t launch_chain<true, 1>(int, int, const int *, size_t, cudaStream_t,
                                               const SysDev *, ChainHdr *, const ChainArrays &,
                                               MoveCtx *, LogRec *, int, int, int,
                                               const double *, const WidomJob &);
template cudaError_t set_chain_smem<true, 1>(size_t);
template cudaError_t max_clusters<true, 1>(int, size_t, int *);
}  // namespace fmc
