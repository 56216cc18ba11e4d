// Host-only check of the tensor-core operand layout (wotg_tc.cuh): the packed
// tile offsets core_offset(r, k, K) are a bijection of 128 rows x K halfs onto
// the tile's 256 K bytes, and the shared-memory descriptors the MMA issuer
// builds for each 16-half K step (start + st * 2 * kCoreLbo, LBO = kCoreLbo,
// SBO = K * 16) address exactly those bytes in the no-swizzle core-matrix
// order. Also decodes the instruction descriptor's M and N. Launches nothing.
#include <cstdio>
#include <vector>

#include "wotg_tc.cuh"

using namespace wotg;

static int check_layout(int K) {
  std::vector<int> hit(128 * K * 2, 0);
  for (int r = 0; r < 128; ++r)
    for (int k = 0; k < K; ++k) {
      const uint32_t b = tc::core_offset(r, k, K);
      if (b % 2 || b + 2 > (uint32_t)(128 * K * 2)) return 1;   // inside the tile, half-aligned
      if (hit[b]++) return 2;                                     // no two elements share bytes
    }
  const uint32_t base = 0x1000;                                   // any 16-byte aligned start
  for (int st = 0; st < K / 16; ++st) {
    const uint64_t d = tc::smem_desc(base + (uint32_t)st * 2u * tc::kCoreLbo, tc::kCoreLbo, (uint32_t)K * 16u);
    const uint32_t start = (uint32_t)(d & 0x3FFFu) << 4;
    const uint32_t lbo = (uint32_t)((d >> 16) & 0x3FFFu) << 4;
    const uint32_t sbo = (uint32_t)((d >> 32) & 0x3FFFu) << 4;
    if (((d >> 46) & 7u) != 1u || (d >> 61) != 0u) return 3;    // fixed bits, no swizzle
    for (int r = 0; r < 128; ++r)
      for (int kk = 0; kk < 16; ++kk) {
        // canonical K-major no-swizzle layout of one 128 x 16 operand slice
        const uint32_t addr = start + (uint32_t)(r / 8) * sbo + (uint32_t)(kk / 8) * lbo + (uint32_t)(r % 8) * 16u +
                              (uint32_t)(kk % 8) * 2u;
        if (addr != base + tc::core_offset(r, 16 * st + kk, K)) return 4;
      }
  }
  return 0;
}

int main() {
  for (int K : {32, 64}) {
    const int r = check_layout(K);
    if (r) {
      std::printf("FAIL K=%d code=%d\n", K, r);
      return 1;
    }
  }
  const uint32_t id = tc::idesc_f16_f32(128, 128);
  if (((id >> 17) & 0x3Fu) * 8u != 128u || ((id >> 24) & 0x1Fu) * 16u != 128u || ((id >> 4) & 3u) != 1u) {
    std::printf("FAIL idesc %08x\n", id);
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
