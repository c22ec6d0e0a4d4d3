// Instantiations of the tcgen05 SB kernel for FP16 hi + lo operands (real couplings, scaled by
// powers of two into FP16's range: 22 bits per operand where BF16 hi + lo keeps 16): dSB, and bSB
// with x split too; the dSB energy mode ranks bSB replicas (sign operands against the split couplings).
#include "sb_tc_kernel.cuh"

namespace sbk {

bool tc_kernel_split16(int variant, int nr, int emode, const void **k, size_t *smem) {
  if (variant == 2) {
    switch (nr) {
      case 32: return tck::tc_lookup<kTcFp16Split, 2, 32, 7>(emode, k, smem);
      case 64: return tck::tc_lookup<kTcFp16Split, 2, 64, 7>(emode, k, smem);
      case 128: return tck::tc_lookup<kTcFp16Split, 2, 128, 7>(emode, k, smem);
    }
  }
  if (variant == 1) {
    switch (nr) {
      case 32: return tck::tc_lookup<kTcFp16Split, 1, 32, 1>(emode, k, smem);
      case 64: return tck::tc_lookup<kTcFp16Split, 1, 64, 1>(emode, k, smem);
      case 128: return tck::tc_lookup<kTcFp16Split, 1, 128, 1>(emode, k, smem);
    }
  }
  return false;
}

}  // namespace sbk
