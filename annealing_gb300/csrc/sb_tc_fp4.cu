// Instantiations of the packed-E2M1 tcgen05 dSB kernel (integer |J| <= 4, J resident in shared memory).
#include "sb_tc_fp4.cuh"

namespace sbk {

namespace {
// The whole shared memory of one CTA (dynamic + this kernel's static arrays) must stay within the
// 227 KB an SM grants one block.
constexpr size_t kSmemLimit = 232448;
constexpr size_t kStaticReserve = 4096;

template <int NR, bool PAIR = false>
bool lookup(int emode, int k_chunks, const void **k, size_t *smem) {
  *smem = tck::fp4_smem<NR, PAIR>(k_chunks);
  *k = nullptr;
  if (*smem + kStaticReserve > kSmemLimit) return false;
  if (emode == tck::kEmodeStep) *k = reinterpret_cast<const void *>(&tck::tc_fp4_kernel<NR, tck::kEmodeStep, PAIR>);
  if (emode == tck::kEmodeStepTrace)
    *k = reinterpret_cast<const void *>(&tck::tc_fp4_kernel<NR, tck::kEmodeStepTrace, PAIR>);
  if (emode == tck::kEmodeEnergy) *k = reinterpret_cast<const void *>(&tck::tc_fp4_kernel<NR, tck::kEmodeEnergy, PAIR>);
  return *k != nullptr;
}
}  // namespace

// k_chunks: 256-spin chunks of K (Kp / 256); false when the unit's J rows do not fit shared memory.
// pair: the CTA-pair form (clusters of two, 128-replica tile only).
bool tc_kernel_fp4(int variant, int nr, int emode, int k_chunks, const void **k, size_t *smem, bool pair) {
  if (variant != 2 || k_chunks <= 0) return false;
  if (pair) return nr == 128 && lookup<128, true>(emode, k_chunks, k, smem);
  switch (nr) {
    case 32: return lookup<32>(emode, k_chunks, k, smem);
    case 64: return lookup<64>(emode, k_chunks, k, smem);
    case 128: return lookup<128>(emode, k_chunks, k, smem);
  }
  return false;
}

}  // namespace sbk
