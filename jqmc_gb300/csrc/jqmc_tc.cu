// The dense lambda-GEMM of the mixed-precision table rebuild on the fifth-
// generation tensor cores (sm_103a): M = Phi L with Phi the AO values of a tile
// of 128 electrons (FP64) and L the geminal's AO pairing matrix lambda (spin up)
// or its transpose (spin down), jqmc/determinant.py:1380-1402.
//
// The rebuild needs M to about 1e-13 relative, far beyond bf16 or tf32.  Each
// operand row (column) is scaled by a power of two into (-1, 1) and split into
// six 8-bit integer slices (Ozaki's error-free splitting); a bf16 holds each slice
// exactly, every slice product is an exact 16-bit integer, and sums of at most
// 2^24 / 2^14 = 1024 such products are exact in the FP32 accumulators.  The
// products of slice pairs (s, t) with s + t <= 5 (slice s stored as its integer
// times 2^-8s, so a product carries the scale of its level) are accumulated per
// level d = s + t in tensor memory (TMEM):
//   level 0           one accumulator over all of K (K <= 768)
//   level 1 (2 pairs) one accumulator per 512 of K
//   level 2 (3 pairs) one accumulator per 256 of K
//   level 3 (4 pairs) one accumulator; levels 4, 5 one more (the accumulators
//                     round toward zero once a sum passes 2^24: about 2^-40 of
//                     the total for level 3, far less for 4 and 5)
// so eight 128 x 64 FP32 accumulators fill the 512 TMEM columns of the SM.  The
// epilogue reads them back with tcgen05.ld, adds the levels as float-float pairs
// and scales by the row and column exponents.
//
// Data movement: the sliced operands are laid out in global memory exactly as the
// tensor cores read them from shared memory (canonical K-major core matrices, no
// swizzle), so each K chunk of a tile is two contiguous blocks fetched by the TMA
// engine (cp.async.bulk) into a three-stage ring; one thread issues the copies
// and the MMAs, and mbarriers carry the completions (copies -> MMA, MMA -> reuse
// of the stage).  Every wait is bounded: a wait that runs out marks the tile's
// walkers, writes NaN to its outputs, frees TMEM and returns.

#include "jqmc_tc.h"

namespace jqmc_tc {
namespace {

constexpr int kAcc = 8;
constexpr int kTmemCols = kAcc * kBN;   // 512
constexpr unsigned long long kWaitNs = 2000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, unsigned parity) {
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

// Wait for the phase of the given parity; false after about 2 s.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  if (mbar_test(bar, parity)) return true;
  const unsigned long long t0 = now_ns();
  while (!mbar_test(bar, parity))
    if (now_ns() - t0 > kWaitNs) return false;
  return true;
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// Shared-memory matrix descriptor: K-major, no swizzle; lbo = byte distance of
// K-adjacent core matrices, sbo = of 8-row groups; bit 46 = descriptor version.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, bf16 A and B, both
// K-major, N = kBN, M = kBM.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kBN >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);

__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"((uint32_t)accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// The 16 columns at taddr of all eight accumulators (acc j at column j * kBN),
// for this thread's TMEM lane.  The loads and tcgen05.wait::ld are one asm
// statement: tcgen05.ld is asynchronous, so its destination registers may be
// read only after the wait, and the compiler must not move them before it.
__device__ __forceinline__ void tmem_ld_acc(uint32_t taddr, float (*v)[16]) {
  uint32_t r[128];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%128];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%129];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47}, [%130];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63}, [%131];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%64, %65, %66, %67, %68, %69, %70, %71, %72, %73, %74, %75, %76, %77, %78, %79}, [%132];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%80, %81, %82, %83, %84, %85, %86, %87, %88, %89, %90, %91, %92, %93, %94, %95}, [%133];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%96, %97, %98, %99, %100, %101, %102, %103, %104, %105, %106, %107, %108, %109, %110, %111}, [%134];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%112, %113, %114, %115, %116, %117, %118, %119, %120, %121, %122, %123, %124, %125, %126, %127}, [%135];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]),
        "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]),
        "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]),
        "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]),
        "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63]),
        "=r"(r[64]), "=r"(r[65]), "=r"(r[66]), "=r"(r[67]), "=r"(r[68]), "=r"(r[69]), "=r"(r[70]), "=r"(r[71]),
        "=r"(r[72]), "=r"(r[73]), "=r"(r[74]), "=r"(r[75]), "=r"(r[76]), "=r"(r[77]), "=r"(r[78]), "=r"(r[79]),
        "=r"(r[80]), "=r"(r[81]), "=r"(r[82]), "=r"(r[83]), "=r"(r[84]), "=r"(r[85]), "=r"(r[86]), "=r"(r[87]),
        "=r"(r[88]), "=r"(r[89]), "=r"(r[90]), "=r"(r[91]), "=r"(r[92]), "=r"(r[93]), "=r"(r[94]), "=r"(r[95]),
        "=r"(r[96]), "=r"(r[97]), "=r"(r[98]), "=r"(r[99]), "=r"(r[100]), "=r"(r[101]), "=r"(r[102]), "=r"(r[103]),
        "=r"(r[104]), "=r"(r[105]), "=r"(r[106]), "=r"(r[107]), "=r"(r[108]), "=r"(r[109]), "=r"(r[110]), "=r"(r[111]),
        "=r"(r[112]), "=r"(r[113]), "=r"(r[114]), "=r"(r[115]), "=r"(r[116]), "=r"(r[117]), "=r"(r[118]), "=r"(r[119]),
        "=r"(r[120]), "=r"(r[121]), "=r"(r[122]), "=r"(r[123]), "=r"(r[124]), "=r"(r[125]), "=r"(r[126]), "=r"(r[127])
      : "r"(taddr + 0 * kBN), "r"(taddr + 1 * kBN), "r"(taddr + 2 * kBN), "r"(taddr + 3 * kBN), "r"(taddr + 4 * kBN), "r"(taddr + 5 * kBN), "r"(taddr + 6 * kBN), "r"(taddr + 7 * kBN)
      : "memory");
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int x = 0; x < 16; ++x) v[j][x] = __uint_as_float(r[16 * j + x]);
}

__device__ __forceinline__ void two_sum(float& h, float& l, float x) {
  const float t = __fadd_rn(h, x);
  const float z = __fsub_rn(t, h);
  l += __fadd_rn(__fsub_rn(h, __fsub_rn(t, z)), __fsub_rn(x, z));
  h = t;
}

// Accumulator of slice level d for K chunk c (kKC = 32 columns of K per chunk).
__device__ __forceinline__ int acc_of(int d, int c) {
  if (d == 0) return 0;
  if (d == 1) return 1 + (c >= 16 ? 1 : 0);
  if (d == 2) return 3 + (c >> 3);
  if (d == 3) return 6;
  return 7;
}

__global__ void __launch_bounds__(128, 1)
    k_ozaki_m(const uint8_t* __restrict__ a_sl, const uint8_t* __restrict__ b_sl, const int* __restrict__ row_exp,
              const int* __restrict__ col_exp, int nk, long long row0, long long rows_total, int n, int ncols, int slot,
              unsigned used, float2* __restrict__ out, int* status, int fail_bit) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* stage_a = smem;                                  // kStages x kAStage
  uint8_t* stage_b = smem + kStages * kAStage;              // kStages x kBStage
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * (kAStage + kBStage));
  uint64_t* full = bars;                 // kStages: the stage's copies landed
  uint64_t* empty = bars + kStages;      // kStages: the MMAs reading the stage finished
  uint64_t* done = bars + 2 * kStages;   // every MMA issued finished
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kStages + 1);
  int* fail = reinterpret_cast<int*>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5;
  const int ct = blockIdx.x, rt = blockIdx.y;
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  const uint8_t* a_tile = a_sl + (size_t)rt * nk * kAStage;
  const uint8_t* b_tile = b_sl + (size_t)ct * nk * kBStage;
  if (tid == 0) {
    int issued[kStages] = {}, landed[kStages] = {};   // copies per stage, and waited for
    auto load = [&](int c) {
      const int s = c % kStages;
      ++issued[s];
      mbar_arrive_expect_tx(&full[s], kAStage + kBStage);
      bulk_load(stage_a + s * kAStage, a_tile + (size_t)c * kAStage, kAStage, &full[s]);
      bulk_load(stage_b + s * kBStage, b_tile + (size_t)c * kBStage, kBStage, &full[s]);
    };
    for (int c = 0; c < nk && c < kStages; ++c) load(c);
    unsigned init = 0;   // accumulators written so far
    bool ok = true;
    for (int c = 0; c < nk && ok; ++c) {
      const int s = c % kStages;
      if (!mbar_wait(&full[s], (c / kStages) & 1)) { ok = false; break; }
      ++landed[s];
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a0 = smem_u32(stage_a + s * kAStage), b0 = smem_u32(stage_b + s * kBStage);
#pragma unroll
      for (int ks = 0; ks < kKC / 16; ++ks) {
#pragma unroll
        for (int sa = 0; sa < kSlices; ++sa) {
#pragma unroll
          for (int sb = 0; sb + sa < kSlices; ++sb) {
            const int j = acc_of(sa + sb, c);
            const uint64_t ad = smem_desc(a0 + sa * kASliceBytes + ks * 256, 128, 512);
            const uint64_t bd = smem_desc(b0 + sb * kBSliceBytes + ks * 256, 128, 512);
            mma(tmem + j * kBN, ad, bd, (init >> j) & 1u);
            init |= 1u << j;
          }
        }
      }
      mma_commit(&empty[s]);
      // refill the stage of the previous chunk once its MMAs are done (those of
      // this chunk are queued behind them, so the tensor pipe stays busy)
      if (c >= 1 && c - 1 + kStages < nk) {
        const int sp = (c - 1) % kStages;
        if (!mbar_wait(&empty[sp], ((c - 1) / kStages) & 1)) { ok = false; break; }
        load(c - 1 + kStages);
      }
    }
    // completes when every MMA issued above has finished (also on the error path,
    // so that TMEM is released only after them)
    mma_commit(done);
    if (!ok) {
      *fail = 1;
      // let every copy issued so far land before the shared memory is released
      for (int s = 0; s < kStages; ++s)
        for (; landed[s] < issued[s]; ++landed[s])
          if (!mbar_wait(&full[s], landed[s] & 1)) break;
    }
  }
  __syncthreads();
  const bool fin = mbar_wait(done, 0);
  const bool ok = __syncthreads_and(fin && *fail == 0) != 0;   // uniform: tcgen05.ld is warp-collective
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  // epilogue: thread t owns row t of the tile (TMEM lane t)
  const long long g = row0 + (long long)rt * kBM + tid;
  const bool row_ok = g < rows_total;
  const int w = row_ok ? (int)(g / n) : 0, i = row_ok ? (int)(g % n) : 0;
  float2* orow = out + ((size_t)w * 2 + slot) * (size_t)n * ncols + (size_t)i * ncols;
  const int rexp = row_ok ? row_exp[g - row0] : 0;
  const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
  const float nan = __int_as_float(0x7fc00000);
#pragma unroll 1
  for (int q = 0; q < kBN / 16; ++q) {
    float v[kAcc][16];
    if (ok) tmem_ld_acc(lane_base + q * 16, v);   // (warp-uniform condition)
#pragma unroll
    for (int j = 0; j < kAcc; ++j)   // accumulators no MMA wrote hold no data
#pragma unroll
      for (int x = 0; x < 16; ++x) v[j][x] = (ok && ((used >> j) & 1u)) ? v[j][x] : 0.f;
    if (!row_ok) continue;
#pragma unroll
    for (int x = 0; x < 16; ++x) {
      const int b = ct * kBN + q * 16 + x;
      if (b >= ncols) break;
      float h = v[0][x], l = 0.f;   // (the slices carry their levels' scales)
#pragma unroll
      for (int j = 1; j < kAcc; ++j) two_sum(h, l, v[j][x]);
      const float hs = __fadd_rn(h, l);   // renormalise the pair
      const float ls = __fadd_rn(__fsub_rn(h, hs), l);
      const float sc = ldexpf(1.0f, rexp + col_exp[b] - 14);
      orow[b] = ok ? make_float2(hs * sc, ls * sc) : make_float2(nan, nan);
    }
  }
  if (!ok && row_ok && status) atomicOr(status + w, fail_bit);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

}  // namespace

int ozaki_gemm(const uint16_t* a_slices, const uint16_t* b_slices, const int* row_exp, const int* col_exp, int nk_chunks,
               int n_col_tiles, int row_tiles, long long row0, long long rows_total, int n, int ncols, int slot, float2* out,
               int* status, int fail_bit, cudaStream_t stream) {
  if (nk_chunks <= 0 || nk_chunks * kKC > kMaxK || n_col_tiles <= 0 || row_tiles <= 0) return -1;
  static bool attr_set[64] = {false};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -3;
  if (!attr_set[dev]) {
    if (cudaFuncSetAttribute(k_ozaki_m, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes) != cudaSuccess) return -3;
    attr_set[dev] = true;
  }
  unsigned used = 1u | (1u << 1) | (1u << 6) | (1u << 7);
  if (nk_chunks > 16) used |= 1u << 2;
  for (int q = 0; q < 3; ++q)
    if (nk_chunks > 8 * q) used |= 1u << (3 + q);
  const dim3 grid(n_col_tiles, row_tiles);
  k_ozaki_m<<<grid, 128, kSmemBytes, stream>>>(reinterpret_cast<const uint8_t*>(a_slices),
                                                 reinterpret_cast<const uint8_t*>(b_slices), row_exp, col_exp, nk_chunks,
                                                 row0, rows_total, n, ncols, slot, used, out, status, fail_bit);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

}  // namespace jqmc_tc
