// gbsp_pass1.cu -- pass-1 kernels with recurrence twiddles (the default) and
// the host launch functions of both phase modes (gbsp_launch.h).
#include "gbsp_pass1_impl.cuh"

namespace gbsp {

template struct Pass1Set<false>;

int p1_blocks_per_sm(const P1Kernel& k, size_t smem, int* nb) {
    return k.exact ? Pass1Set<true>::blocks(k, smem, nb) : Pass1Set<false>::blocks(k, smem, nb);
}

int p1_launch(const P1Kernel& k, int grid, size_t smem, cudaStream_t st, const P1Args& a) {
    return k.exact ? Pass1Set<true>::launch(k, grid, smem, st, a) : Pass1Set<false>::launch(k, grid, smem, st, a);
}

int p1_batch_blocks_per_sm(const P1Kernel& k, size_t smem, int* nb) {
    return k.exact ? Pass1Set<true>::batch_blocks(k, smem, nb) : Pass1Set<false>::batch_blocks(k, smem, nb);
}

int p1_batch_launch(const P1Kernel& k, int grid, size_t smem, cudaStream_t st, const P1Args* args,
                    const long* item_begin, int nmat, unsigned long long* queue) {
    return k.exact ? Pass1Set<true>::batch_launch(k, grid, smem, st, args, item_begin, nmat, queue)
                   : Pass1Set<false>::batch_launch(k, grid, smem, st, args, item_begin, nmat, queue);
}

}  // namespace gbsp
