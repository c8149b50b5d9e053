// gbsp_pass1_impl.cuh -- compiled pass-1 kernels (k_twiddle_sum and its
// batched form) behind host launch functions, one set per phase mode:
// Pass1Set<false> (twiddles by recurrence, reseeded exactly every 4 rows) is
// instantiated in gbsp_pass1.cu, Pass1Set<true> (every twiddle an exact
// table lookup) in gbsp_pass1_exact.cu, so the two compile in parallel.
// One instance per (index width, twiddle-table layout, 64-bit phases, rows
// per lane); 16-bit indices only occur with rows <= 65536, so never with
// 64-bit phase products.
#pragma once
#include "gbsp_launch.h"

namespace gbsp {

template <typename IDX, int TAB, bool BIG, int KU, bool EXACT>
struct P1Ops {
    static int blocks(size_t smem, int* nb) {
        auto kern = k_twiddle_sum<IDX, TAB, BIG, KU, EXACT>;
        if (int rc = allow_full_smem((const void*)kern)) return rc;
        GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(nb, kern, P1_THREADS, smem));
        return GBSP_OK;
    }
    static int launch(int grid, size_t smem, cudaStream_t st, const P1Args& a) {
        k_twiddle_sum<IDX, TAB, BIG, KU, EXACT><<<grid, P1_THREADS, smem, st>>>(a);
        GB_CUDA(cudaGetLastError());
        return GBSP_OK;
    }
    static int batch_blocks(size_t smem, int* nb) {
        auto kern = k_twiddle_sum_batch<IDX, TAB, BIG, KU, EXACT>;
        if (int rc = allow_full_smem((const void*)kern)) return rc;
        GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(nb, kern, P1_THREADS, smem));
        return GBSP_OK;
    }
    static int batch_launch(int grid, size_t smem, cudaStream_t st, const P1Args* args, const long* item_begin,
                            int nmat, unsigned long long* queue) {
        k_twiddle_sum_batch<IDX, TAB, BIG, KU, EXACT><<<grid, P1_THREADS, smem, st>>>(args, item_begin, nmat, queue);
        GB_CUDA(cudaGetLastError());
        return GBSP_OK;
    }
};

// Calls f(Ops{}) with the P1Ops instance of k.
template <bool EXACT, typename F>
int with_p1(const P1Kernel& k, F&& f) {
    auto by_ku = [&](auto idx_tag, auto tab_tag, auto big_tag) {
        using IDX = decltype(idx_tag);
        constexpr int TAB = decltype(tab_tag)::value;
        constexpr bool BIG = decltype(big_tag)::value;
        return k.ku == 8 ? f(P1Ops<IDX, TAB, BIG, 8, EXACT>{}) : f(P1Ops<IDX, TAB, BIG, 4, EXACT>{});
    };
    auto by_idx = [&](auto tab_tag) {
        if (k.idx_bytes == 2) return by_ku(uint16_t{}, tab_tag, std::false_type{});
        if (k.big) return by_ku(uint32_t{}, tab_tag, std::true_type{});
        return by_ku(uint32_t{}, tab_tag, std::false_type{});
    };
    switch (k.tab) {
        case TAB_HALF: return by_idx(std::integral_constant<int, TAB_HALF>{});
        case TAB_TWO: return by_idx(std::integral_constant<int, TAB_TWO>{});
        default: return by_idx(std::integral_constant<int, TAB_FULL>{});
    }
}

template <bool EXACT>
struct Pass1Set {
    static int blocks(const P1Kernel& k, size_t smem, int* nb) {
        return with_p1<EXACT>(k, [&](auto ops) { return decltype(ops)::blocks(smem, nb); });
    }
    static int launch(const P1Kernel& k, int grid, size_t smem, cudaStream_t st, const P1Args& a) {
        return with_p1<EXACT>(k, [&](auto ops) { return decltype(ops)::launch(grid, smem, st, a); });
    }
    static int batch_blocks(const P1Kernel& k, size_t smem, int* nb) {
        return with_p1<EXACT>(k, [&](auto ops) { return decltype(ops)::batch_blocks(smem, nb); });
    }
    static int batch_launch(const P1Kernel& k, int grid, size_t smem, cudaStream_t st, const P1Args* args,
                            const long* item_begin, int nmat, unsigned long long* queue) {
        return with_p1<EXACT>(k, [&](auto ops) {
            return decltype(ops)::batch_launch(grid, smem, st, args, item_begin, nmat, queue);
        });
    }
};

extern template struct Pass1Set<false>;
extern template struct Pass1Set<true>;

}  // namespace gbsp
