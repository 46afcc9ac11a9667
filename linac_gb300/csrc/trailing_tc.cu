// Tensor-core trailing update for 32-bit residues (placeholder until the
// tcgen05 limb kernel lands): reports itself unavailable so the driver uses
// the SIMT contraction.
#include "rref_internal.cuh"

namespace lnc {

bool trailing_tc_u32_available() { return false; }
size_t trailing_tc_u32_scratch(int64_t, int64_t, int) { return 0; }
int trailing_update_tc_u32(const TrailingCtx<FieldU32>& t, cudaStream_t s) {
    return trailing_update_simt<FieldU32>(t, s);
}

}  // namespace lnc
