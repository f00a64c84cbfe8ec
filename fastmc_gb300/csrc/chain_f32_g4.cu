// chain_f32_g4.cu -- one instantiation of the chain kernel (F32 = true, GN = kMaxG).
#include "chain_kernel.cuh"

namespace fmc {
template cudaError_t launch_chain<true, kMaxG>(int, int, const int *, size_t, cudaStream_t,
                                               const SysDev *, ChainHdr *, const ChainArrays &,
                                               MoveCtx *, LogRec *, int, int, int,
                                               const double *, const WidomJob &);
template cudaError_t set_chain_smem<true, kMaxG>(size_t);
template cudaError_t max_clusters<true, kMaxG>(int, size_t, int *);
}  // namespace fmc
