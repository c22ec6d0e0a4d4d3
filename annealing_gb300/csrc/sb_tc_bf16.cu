// Instantiations of the tcgen05 SB kernel for BF16 operands (dSB, integer |J| <= 256; NMFA, integer
// |J| <= 256 against the BF16 hi + lo state).
#include "sb_tc_kernel.cuh"

namespace sbk {

bool tc_kernel_bf16(int variant, int nr, int emode, const void **k, size_t *smem) {
  if (variant == 2) {
    switch (nr) {
      case 32: return tck::tc_lookup<kTcBf16, 2, 32, 7>(emode, k, smem);
      case 64: return tck::tc_lookup<kTcBf16, 2, 64, 7>(emode, k, smem);
      case 128: return tck::tc_lookup<kTcBf16, 2, 128, 7>(emode, k, smem);
    }
  }
  if (variant == 3) {
    switch (nr) {
      case 32: return tck::tc_lookup<kTcBf16, 3, 32, 1>(emode, k, smem);
      case 64: return tck::tc_lookup<kTcBf16, 3, 64, 1>(emode, k, smem);
      case 128: return tck::tc_lookup<kTcBf16, 3, 128, 1>(emode, k, smem);
    }
  }
  return false;
}

}  // namespace sbk
