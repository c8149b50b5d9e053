// gbsp_pass1_exact.cu -- pass-1 kernels whose every twiddle is read from the
// shared-memory table at its exact integer phase (gbsp_options.exact_phases).
#include "gbsp_pass1_impl.cuh"

namespace gbsp {

template struct Pass1Set<true>;

}  // namespace gbsp
