// Device helpers shared by the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "svm_internal.h"

namespace svm {

// ---------------------------------------------------------------- mbarrier / bulk copy (PTX)
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for phase `parity` of `bar` to complete, giving up after `limit`
// polls (try_wait itself blocks for a hardware-defined interval per poll).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit) {
  for (uint32_t n = 0; n < limit; n++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// A ring position: the stage of the current tile and the parity of that
// stage's current use, advanced tile by tile, so that no loop divides its
// 64-bit tile count by the run-time ring depth.
struct RingPos {
  int s = 0;
  uint32_t phase = 0;
  __device__ __forceinline__ void next(int nst) {
    if (++s == nst) {
      s = 0;
      phase ^= 1u;
    }
  }
};

// 1-D bulk copy global -> shared, completion signalled as transaction bytes on `bar`.
// dst and src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void raise_error(int* err, int code) {
  if (err) atomicCAS(err, 0, code);
}

// One int32 C-expression program over an operand array (see ExprOp).
__device__ __forceinline__ int32_t apply_bin_dev(int op, int32_t a, int32_t b, bool& div0) {
  uint32_t ua = (uint32_t)a, ub = (uint32_t)b;
  switch (op) {
    case X_ADD: return (int32_t)(ua + ub);
    case X_SUB: return (int32_t)(ua - ub);
    case X_MUL: return (int32_t)(ua * ub);
    case X_DIV:
      if (b == 0) { div0 = true; return 0; }
      if (a == INT32_MIN && b == -1) return INT32_MIN;
      return a / b;
    case X_MOD:
      if (b == 0) { div0 = true; return 0; }
      if (b == -1) return 0;
      return a % b;
    case X_SHL: return (int32_t)(ua << (ub & 31));
    case X_SHR: return a >> (ub & 31);
    case X_LT: return a < b;
    case X_LE: return a <= b;
    case X_GT: return a > b;
    case X_GE: return a >= b;
    case X_EQ: return a == b;
    case X_NE: return a != b;
    case X_BAND: return a & b;
    case X_BXOR: return a ^ b;
    case X_BOR: return a | b;
  }
  return 0;
}

static __device__ __noinline__ int32_t eval_prog(const Prog& p, const int32_t* opnd, int* err) {
  int32_t st[16];
  int sp = 0;
  bool div0 = false;
  for (int pc = 0; pc < p.n;) {
    int op = p.op[pc], arg = p.arg[pc];
    pc++;
    switch (op) {
      case X_OPND: st[sp++] = opnd[arg]; break;
      case X_CONST: st[sp++] = p.konst[arg]; break;
      case X_NEG: st[sp - 1] = (int32_t)(0u - (uint32_t)st[sp - 1]); break;
      case X_NOT: st[sp - 1] = !st[sp - 1]; break;
      case X_BNOT: st[sp - 1] = ~st[sp - 1]; break;
      case X_NORM: st[sp - 1] = st[sp - 1] != 0; break;
      case X_JZ_KEEP: if (st[sp - 1] == 0) pc = arg; else sp--; break;
      case X_JNZ_ONE: if (st[sp - 1] != 0) { st[sp - 1] = 1; pc = arg; } else sp--; break;
      case X_JZ_POP: if (st[--sp] == 0) pc = arg; break;
      case X_JMP: pc = arg; break;
      default: {
        int32_t b = st[--sp];
        st[sp - 1] = apply_bin_dev(op, st[sp - 1], b, div0);
      }
    }
  }
  if (div0) raise_error(err, DERR_DIV0);
  return sp ? st[sp - 1] : 0;
}

// ---------------------------------------------------------------- dimension probe
// Looks `key` up in table d (global, or staged in shared memory at smem_base).
// On success returns true and the entry (bit 0 = present, payload above).
__device__ __forceinline__ bool probe_dim(const DimDesc& d, const uint32_t* smem_base, int32_t key,
                                          uint32_t& entry) {
  const uint32_t* w = d.smem_word_off >= 0 ? smem_base + d.smem_word_off : d.words;
  bool in_smem = d.smem_word_off >= 0;
  if (d.layout == LAYOUT_DENSE) {
    uint32_t idx = (uint32_t)key - (uint32_t)d.key_min;
    if (idx >= d.span) return false;
    uint64_t bit = (uint64_t)idx * (uint32_t)d.entry_bits;
    uint32_t word = in_smem ? w[bit >> 5] : __ldg(w + (bit >> 5));
    uint32_t e = d.entry_bits == 32 ? word : (word >> (bit & 31)) & ((1u << d.entry_bits) - 1u);
    entry = e;
    return (e & 1u) != 0;
  }
  uint32_t mask = d.span - 1u;
  uint32_t slot = mix32((uint32_t)key) & mask;
  for (uint32_t n = 0; n <= mask; n++) {
    uint2 kv = in_smem ? reinterpret_cast<const uint2*>(w)[slot]
                       : __ldg(reinterpret_cast<const uint2*>(w) + slot);
    if (kv.y == 0u) return false;
    if ((int32_t)kv.x == key) {
      entry = kv.y;
      return true;
    }
    slot = (slot + 1u) & mask;
  }
  return false;
}

__device__ __forceinline__ int32_t payload_value(const DimDesc& d, int f, uint32_t entry) {
  const PayloadField& p = d.pay[f];
  uint32_t v = p.bits == 0 ? 0u : (p.bits >= 32 ? entry >> p.shift : (entry >> p.shift) & ((1u << p.bits) - 1u));
  if (p.col) return __ldg(p.col + v);
  return (int32_t)((uint32_t)p.min + v);
}

// ---------------------------------------------------------------- hashing
// The reference's key hash (com/cpp/cpu-runtime.hpp:68-74) over the 4
// little-endian bytes of an int key: h = h*31 + byte, then clear bit 31.
__host__ __device__ __forceinline__ uint32_t ref_hash_i32(int32_t key, int signed_char) {
  uint32_t h = 0;
  uint32_t k = (uint32_t)key;
  for (int i = 0; i < 4; i++) {
    int b = (int)((k >> (8 * i)) & 0xFFu);
    if (signed_char && b >= 128) b -= 256;
    h = h * 31u + (uint32_t)b;
  }
  return h & 0x7FFFFFFFu;
}

// splitmix64 output function (Steele, Lea, Flood 2014) applied to z + golden.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace svm
