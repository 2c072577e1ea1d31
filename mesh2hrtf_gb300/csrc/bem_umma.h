// bem_umma.h - encodings of the 5th-generation tensor-core (tcgen05)
// operands used by the shared-matrix product: the instruction descriptor and
// the shared-memory matrix descriptor, as the PTX ISA defines them for
// tcgen05.mma (sm_100 family).  Plain constexpr C++ so that host tests can
// check every field; the functions are also callable in device code.
//
// Instruction descriptor (32 bits) of .kind::tf32 / .kind::f16:
//   [0,2) sparsity selector  [2] sparsity  [3] saturate
//   [4,6) D format (0 F16, 1 F32)          [6] reserved
//   [7,10) A format  [10,13) B format (kind::f16: 0 F16, 1 BF16;
//                                      kind::tf32: 2 TF32)
//   [13] negate A  [14] negate B  [15] A major (0 K)  [16] B major (0 K)
//   [17,23) N >> 3  [23] reserved  [24,29) M >> 4  [29] reserved
//   [30,32) maximum shift (.ws only)
//
// Shared-memory matrix descriptor (64 bits):
//   [0,14)  start address >> 4
//   [16,30) leading-dimension byte offset >> 4
//   [32,46) stride-dimension byte offset >> 4
//   [46,48) version (1 on sm_100)
//   [49,52) base offset (0: tiles aligned to the swizzle pattern)
//   [52]    leading-offset mode (0 relative)
//   [61,64) layout: 0 no swizzle, 1 128-byte swizzle with 32-byte atoms,
//           2 128-byte swizzle, 4 64-byte swizzle, 6 32-byte swizzle
// For a K-major operand with the 128-byte swizzle, a row holds 128 bytes of
// K, 8 rows form one 1024-byte swizzle atom, the stride offset is the
// distance between 8-row groups (1024 bytes when the atoms are stacked
// along M / N), and the leading offset is unused (encoded as 1); successive
// K steps inside the 128-byte row advance the start address by the step's
// bytes (32 bytes for K = 8 TF32 values).
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define BEM_UMMA_HD __host__ __device__
#else
#define BEM_UMMA_HD
#endif

namespace bem {
namespace umma {

enum : uint32_t { kFmtF16 = 0, kFmtBF16 = 1, kFmtTF32 = 2 };
enum : uint32_t { kDF16 = 0, kDF32 = 1 };
enum : uint32_t { kLayoutNone = 0, kLayout128B = 2, kLayout64B = 4, kLayout32B = 6 };

BEM_UMMA_HD constexpr uint32_t instr_desc(uint32_t d_fmt, uint32_t a_fmt, uint32_t b_fmt, uint32_t m, uint32_t n,
                              bool a_mn_major = false, bool b_mn_major = false) {
    return (d_fmt << 4) | (a_fmt << 7) | (b_fmt << 10) | ((a_mn_major ? 1u : 0u) << 15) |
           ((b_mn_major ? 1u : 0u) << 16) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

BEM_UMMA_HD constexpr uint64_t smem_desc(uint32_t addr, uint32_t lbo_bytes, uint32_t sbo_bytes, uint32_t layout) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo_bytes >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo_bytes >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46) | ((uint64_t)(layout & 7u) << 61);
}

// the descriptor of the same operand K bytes further along its rows (inside
// one 128-byte swizzled row)
BEM_UMMA_HD constexpr uint64_t smem_desc_advance(uint64_t desc, uint32_t k_bytes) { return desc + (uint64_t)(k_bytes >> 4); }

// Byte offset of element (row, 4-byte column c < 32) inside a K-major tile
// with the 128-byte swizzle: rows of 128 bytes, the 16-byte chunk index
// XORed with the row's position in its 8-row atom (the layout TMA writes
// with CU_TENSOR_MAP_SWIZZLE_128B into a 1024-byte aligned tile).
BEM_UMMA_HD constexpr uint32_t sw128_offset(uint32_t row, uint32_t c) {
    return row * 128u + ((((c * 4u) >> 4) ^ (row & 7u)) << 4) + ((c * 4u) & 15u);
}

// TMEM address of (lane, column): lane in bits [16,32), column in [0,16)
BEM_UMMA_HD constexpr uint32_t tmem_addr(uint32_t base, uint32_t lane, uint32_t col) { return base + (lane << 16) + col; }

}  // namespace umma
}  // namespace bem
