// 64x64 carry-less product by the Arm PMULL instruction for the host-side
// GF(2^128) arithmetic (host_field.h), on Arm hosts built with the crypto
// extension (build.py passes -march=armv8-a+crypto there). Elsewhere this file
// is empty and host_field.h uses its portable product.
#include <cstdint>

#if defined(__aarch64__) && (defined(__ARM_FEATURE_AES) || defined(__ARM_FEATURE_CRYPTO))
#include <arm_neon.h>

void flock_host_clmul64(uint64_t a, uint64_t b, uint64_t* lo, uint64_t* hi) {
  const uint64x2_t v = vreinterpretq_u64_p128(vmull_p64((poly64_t)a, (poly64_t)b));
  *lo = vgetq_lane_u64(v, 0);
  *hi = vgetq_lane_u64(v, 1);
}
#endif
