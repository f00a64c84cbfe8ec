// chain_f64.cu -- one instantiation of the chain kernel (F32 = false, GN = kMaxG).
#include "chain_kernel.cuh"

namespace fmc {
template cudaError_t launch_chain<false, kMaxG>(int, int, const int *, size_t, cudaStream_t,
                                               const SysDev *, ChainHdr *, const ChainArrays &,
                                               MoveCtx *, LogRec *, int, int, int,
                                               const double *, const WidomJob &);
template cudaError_t set_chain_smem<false, kMaxG>(size_t);
template cudaError_t max_clusters<false, kMaxG>(int, size_t, int *);
}  // namespace fmc
