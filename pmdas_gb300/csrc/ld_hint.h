// ld_hint.h — 16-byte global loads with an L2 prefetch-size hint.
//
// PTX `ld .L2::64B / .L2::128B / .L2::256B` (HINT 0: no qualifier).  A leaf
// record's head (node and box: 48 bytes at D = 4) read with the 64-byte hint
// fetches its two sectors only; without a hint, streams over the 128-byte
// records fetched more.  The "memory" clobber keeps the load ordered with the
// thread's own stores.
#pragma once

#include <cuda_runtime.h>

template <int HINT>
__device__ __forceinline__ float4 ld4_hint(const float* p) {
    float4 v;
    if constexpr (HINT == 64)
        asm volatile("ld.global.L2::64B.v4.f32 {%0,%1,%2,%3}, [%4];"
                     : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p) : "memory");
    else if constexpr (HINT == 128)
        asm volatile("ld.global.L2::128B.v4.f32 {%0,%1,%2,%3}, [%4];"
                     : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p) : "memory");
    else if constexpr (HINT == 256)
        asm volatile("ld.global.L2::256B.v4.f32 {%0,%1,%2,%3}, [%4];"
                     : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p) : "memory");
    else
        v = *reinterpret_cast<const float4*>(p);
    return v;
}

// The first NF floats of a 16-byte aligned record (rounded up to 16-byte
// chunks: the record must extend that far) with the 64-byte hint.
template <int NF>
__device__ __forceinline__ void ld_head64(const float* p, float (&out)[(NF + 3) / 4 * 4]) {
#pragma unroll
    for (int k = 0; k < (NF + 3) / 4; ++k) {
        const float4 v = ld4_hint<64>(p + 4 * k);
        out[4 * k] = v.x;
        out[4 * k + 1] = v.y;
        out[4 * k + 2] = v.z;
        out[4 * k + 3] = v.w;
    }
}
