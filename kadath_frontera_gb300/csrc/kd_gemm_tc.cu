// Trailing update of the mixed-precision LU, C -= A * B, on the tcgen05
// tensor cores in TF32 with FP32 accumulation in tensor memory.
//
// The LU works on a column-major FP32 matrix, so the panel L21 (m x k) is
// contiguous along m.  Both operands are first packed K-major with K padded
// to a multiple of 32 (one 128-byte swizzle row of TF32): At[i][kk] = A(i, kk)
// and Bt[j][kk] = B(kk, j).  Each CTA then owns a 128 x 128 tile of C:
//   1. 128 threads copy the tile's operand rows into shared memory in the
//      128-byte-swizzled K-major layout (16-byte chunk c of row r stored at
//      chunk c ^ (r % 8)), then fence them for the async proxy;
//   2. one thread issues K/8 tcgen05.mma.kind::tf32 (M = 128, N = 128,
//      K = 8 each) accumulating into 128 TMEM columns, and commits to an
//      mbarrier;
//   3. four warps wait on the mbarrier (bounded), read the accumulators with
//      tcgen05.ld (warp w owns lanes 32w..32w+31 = tile rows) and update C
//      with coalesced column-major read-modify-writes.
// K of one panel is at most 128, so the whole K extent of a tile fits in
// shared memory and needs no pipelining; the update is bound by the HBM
// traffic of C.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "kd_gemm_tc.hpp"

namespace kd {

namespace {

constexpr int TC_M = 128;
constexpr int TC_N = 128;
constexpr int TC_KBLK = 32;        // TF32 elements per 128-byte row
constexpr int TC_MAXK = 128;       // largest panel width of the one-tile kernel (all of k in shared memory)
constexpr int TC_MAXK_P = 192;     // largest panel width of the persistent kernel (k streamed by 32-wide blocks)
constexpr int TC_THREADS = 128;
constexpr unsigned TC_TMEM_COLS = 128;
constexpr size_t TC_MIN_SMEM = 56 * 1024;
constexpr long long TC_WAIT_LIMIT = 1LL << 26;  // try_wait polls before giving up

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr & 0x3FFFF) >> 4);   // start address
  d |= static_cast<uint64_t>(1) << 16;                   // leading byte offset (unused with swizzle)
  d |= static_cast<uint64_t>(1024 >> 4) << 32;           // stride byte offset
  d |= static_cast<uint64_t>(1) << 46;                   // version
  d |= static_cast<uint64_t>(2) << 61;                   // SWIZZLE_128B
  return d;
}

// Instruction descriptor: D = F32, A = B = TF32, both K-major, M x N.
__host__ __device__ constexpr uint32_t tf32_idesc(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
         (static_cast<uint32_t>(M >> 4) << 24);
}

// Packs a column-major panel into a K-major, zero-padded buffer:
//   out[r * kpad + kk] = src(r, kk) for r < rows, kk < k; 0 elsewhere.
// src(r, kk) = col_major ? src[kk * ld + r] : src[r * ld + kk].
// out_lo != nullptr: also the TF32 rounding of the remainder (v - hi), so
// that hi + lo carries about 21 significant bits (3xTF32 products).
__global__ void pack_kmajor(const float* __restrict__ src, long long ld, int rows, int k, int col_major,
                            float* __restrict__ out, float* __restrict__ out_lo, int rows_pad, int kpad) {
  long long total = static_cast<long long>(rows_pad) * kpad;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    int r, kk;
    if (col_major) {  // read coalesced along r
      r = static_cast<int>(t % rows_pad);
      kk = static_cast<int>(t / rows_pad);
    } else {          // read coalesced along kk
      kk = static_cast<int>(t % kpad);
      r = static_cast<int>(t / kpad);
    }
    float v = 0.0f;
    if (r < rows && kk < k) v = col_major ? src[static_cast<long long>(kk) * ld + r] : src[static_cast<long long>(r) * ld + kk];
    // round to the nearest TF32 value (the tensor cores would truncate)
    uint32_t rounded;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(rounded) : "f"(v));
    const float hi = __uint_as_float(rounded);
    out[static_cast<long long>(r) * kpad + kk] = hi;
    if (out_lo) {
      uint32_t rlo;
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(rlo) : "f"(v - hi));
      out_lo[static_cast<long long>(r) * kpad + kk] = __uint_as_float(rlo);
    }
  }
}

// Copies rows [row0, row0+128) of a K-major buffer (kpad columns) into
// shared memory, one 128 x 32 swizzled block per 32 K-columns.
__device__ __forceinline__ void load_tile_sw128(const float* __restrict__ src, int row0, int kpad, char* smem) {
  const int nkb = kpad / TC_KBLK;
  const int chunks = 128 * 8 * nkb;  // 16-byte chunks
  for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
    int kb = c / (128 * 8);
    int rem = c % (128 * 8);
    int r = rem / 8;
    int ch = rem % 8;
    const float4* g = reinterpret_cast<const float4*>(src + static_cast<long long>(row0 + r) * kpad + kb * TC_KBLK) + ch;
    float4 v = __ldg(g);
    char* dst = smem + kb * (128 * 128) + r * 128 + ((ch ^ (r & 7)) << 4);
    *reinterpret_cast<float4*>(dst) = v;
  }
}

__global__ void __launch_bounds__(TC_THREADS) tf32_update_kernel(const float* __restrict__ At,
                                                                 const float* __restrict__ Bt, int kpad,
                                                                 float* __restrict__ C, long long ldc, int m, int n,
                                                                 int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte aligned operand area: A blocks then B blocks (16 KiB each)
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int nkb = kpad / TC_KBLK;
  char* sA = base;
  char* sB = base + nkb * (128 * 128);
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_base_sh;
  __shared__ int timed_out;

  const int tile_m = blockIdx.x * TC_M;
  const int tile_n = blockIdx.y * TC_N;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    timed_out = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                 "r"(TC_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  load_tile_sw128(At, tile_m, kpad, sA);
  load_tile_sw128(Bt, tile_n, kpad, sB);
  // make the generic-proxy shared-memory writes visible to the tensor cores
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base_sh;

  if (threadIdx.x == 0) {
    const uint32_t idesc = tf32_idesc(TC_M, TC_N);
    const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
    for (int kb = 0; kb < nkb; kb++) {
      for (int k = 0; k < TC_KBLK / 8; k++) {
        uint64_t ad = sw128_desc(a0 + kb * (128 * 128)) + static_cast<uint64_t>((k * 32) >> 4);
        uint64_t bd = sw128_desc(b0 + kb * (128 * 128)) + static_cast<uint64_t>((k * 32) >> 4);
        uint32_t acc = (kb | k) ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
      }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&mbar))
                 : "memory");
  }
  // bounded wait for the MMAs to land in TMEM
  {
    uint32_t done = 0;
    long long it = 0;
    while (!done) {
      asm volatile(
          "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
          : "=r"(done)
          : "r"(smem_u32(&mbar)), "r"(0));
      if (!done && ++it > TC_WAIT_LIMIT) {
        timed_out = 1;
        break;
      }
    }
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  __syncthreads();
  if (!timed_out) {
    const int row = tile_m + warp * 32 + lane;
    for (int c0 = 0; c0 < TC_N; c0 += 16) {
      uint32_t r[16];
      const uint32_t taddr = tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c0);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < m) {
#pragma unroll
        for (int q = 0; q < 16; q++) {
          int col = tile_n + c0 + q;
          if (col < n) {
            float* p = C + static_cast<long long>(col) * ldc + row;
            *p -= __uint_as_float(r[q]);
          }
        }
      }
    }
  } else if (threadIdx.x == 0) {
    atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS));
}

// ---------------------------------------------------------------------------
// Persistent, warp-specialised version (used when C allows TMA: 16-byte
// aligned base, ldc a multiple of 4 floats).  One CTA per SM walks the
// 128 x 128 tiles of C (tile t -> CTA t % grid):
//   warp 0  producer: TMA loads of the tile's operand blocks (128-byte
//           swizzled, K-major) and of C in 128 x 32 chunks through a ring of
//           four shared-memory slots;
//   warp 1  allocates 256 TMEM columns (two 128-column accumulators) and
//           issues the MMAs of a tile into one accumulator while the
//           epilogue drains the other;
//   warps 2-5 epilogue: per C chunk, tcgen05.ld of 32 accumulator columns,
//           C -= acc in shared memory, TMA store of the chunk.
// Every mbarrier wait gives up after GP_TC_WAIT_NS; the CTA then sets the
// error flag, lets its roles fall out of their loops and frees its TMEM.
// warps: 0 operand producer, 1 MMA issuer, 2-5 epilogue, 6 C producer
constexpr int P_THREADS = 224;
constexpr int P_CSLOTS = 8;                              // most C chunks in flight
constexpr int P_NST = 2;                                 // operand stages (one k-block each)
constexpr int P_CCOLS = 32;                              // columns per C chunk
constexpr int P_CHUNK_BYTES = TC_M * P_CCOLS * 4;        // 16 KiB
constexpr int P_OPBLK_BYTES = 128 * 128;                 // 128 rows x 32 TF32
constexpr unsigned long long P_WAIT_NS = 2000000000ull;  // 2 s
constexpr size_t P_MAX_SMEM = 226 * 1024;  // + 1 KiB static shared memory = the 227 KiB per-CTA limit

__device__ __forceinline__ unsigned long long p_now() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait for phase `parity` of an mbarrier; false when it ran out.
__device__ __forceinline__ bool p_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  uint32_t done = 0;
  unsigned long long t0 = 0;
  for (int spin = 0;; spin++) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (spin == 0) t0 = p_now();
    else if ((spin & 255) == 0 && p_now() - t0 > P_WAIT_NS) return false;
  }
}

__device__ __forceinline__ void p_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void p_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void p_tma_load(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// C is streamed once per update: its loads and stores are marked to leave
// L2 first, so that the operand tiles every CTA re-reads stay resident.
__device__ __forceinline__ uint64_t p_evict_first() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

__device__ __forceinline__ void p_tma_load_stream(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar,
                                                  uint64_t pol) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, {%2, "
      "%3}], [%4], %5;" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar)), "l"(pol)
      : "memory");
}

__device__ __forceinline__ void p_tma_store_stream(const CUtensorMap* map, const void* src, int x, int y,
                                                   uint64_t pol) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group.L2::cache_hint [%0, {%2, %3}], [%1], %4;" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(smem_u32(src)), "r"(x), "r"(y), "l"(pol)
               : "memory");
}

__device__ __forceinline__ void p_tma_store(const CUtensorMap* map, const void* src, int x, int y) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(smem_u32(src)), "r"(x), "r"(y)
               : "memory");
}

__device__ __forceinline__ void tf32_mma(uint32_t d, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
      "l"(ad), "l"(bd), "r"(idesc), "r"(accum));
}

__global__ void __launch_bounds__(P_THREADS, 1)
    tf32_update_persistent(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                           const __grid_constant__ CUtensorMap mapAlo, const __grid_constant__ CUtensorMap mapBlo,
                           const __grid_constant__ CUtensorMap mapC, int nkb, int ntm, int ntiles, int split3,
                           int ncs, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char p_raw[];
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(p_raw) + 1023) & ~uintptr_t(1023));
  // P_NST operand stages, each one k-block of A, B (and their lo parts):
  // the k-blocks of consecutive tiles stream through them
  const int nplanes = split3 ? 4 : 2;
  const int stage_bytes = nplanes * P_OPBLK_BYTES;
  char* sC = base + P_NST * stage_bytes;  // ring of ncs C chunks
  __shared__ uint64_t op_full[P_NST], op_empty[P_NST], acc_full[2], acc_empty[2], c_full[P_CSLOTS],
      c_empty[P_CSLOTS];
  __shared__ uint32_t tmem_base_sh;
  __shared__ int abort_flag, epi_abort;
  volatile int* abort_v = &abort_flag;  // written by one role, polled by the others
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    abort_flag = 0;
    epi_abort = 0;
    for (int i = 0; i < P_NST; i++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&op_full[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&op_empty[i])));
    }
    for (int i = 0; i < 2; i++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&acc_full[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&acc_empty[i])));
    }
    for (int i = 0; i < P_CSLOTS; i++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&c_full[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&c_empty[i])));
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapA)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapB)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapC)) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                 "r"(256));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base_sh;

  if (warp == 0) {
    if (lane == 0) {  // ---------------------------------- operand producer
      int g = 0;  // k-blocks issued so far (all tiles)
      for (int tile = blockIdx.x; tile < ntiles && !*abort_v; tile += gridDim.x) {
        const int tm = tile % ntm, tn = tile / ntm;
        for (int kb = 0; kb < nkb; kb++, g++) {
          const int st = g % P_NST, use = g / P_NST;
          if (use > 0 && !p_wait(&op_empty[st], (use - 1) & 1)) {
            *abort_v = 1;
            break;
          }
          char* sp = base + st * stage_bytes;
          p_expect_tx(&op_full[st], static_cast<uint32_t>(stage_bytes));
          p_tma_load(sp, &mapA, kb * TC_KBLK, tm * TC_M, &op_full[st]);
          p_tma_load(sp + P_OPBLK_BYTES, &mapB, kb * TC_KBLK, tn * TC_N, &op_full[st]);
          if (split3) {
            p_tma_load(sp + 2 * P_OPBLK_BYTES, &mapAlo, kb * TC_KBLK, tm * TC_M, &op_full[st]);
            p_tma_load(sp + 3 * P_OPBLK_BYTES, &mapBlo, kb * TC_KBLK, tn * TC_N, &op_full[st]);
          }
        }
      }
    }
  } else if (warp == 6) {
    if (lane == 0) {  // ---------------------------------------- C producer
      const uint64_t pol = p_evict_first();
      int cchunk = 0;
      for (int tile = blockIdx.x; tile < ntiles && !*abort_v; tile += gridDim.x) {
        const int tm = tile % ntm, tn = tile / ntm;
        for (int ch = 0; ch < TC_N / P_CCOLS; ch++, cchunk++) {
          const int slot = cchunk % ncs, use = cchunk / ncs;
          if (use > 0 && !p_wait(&c_empty[slot], (use - 1) & 1)) {
            *abort_v = 1;
            break;
          }
          p_expect_tx(&c_full[slot], P_CHUNK_BYTES);
          p_tma_load_stream(sC + slot * P_CHUNK_BYTES, &mapC, tm * TC_M, tn * TC_N + ch * P_CCOLS, &c_full[slot],
                            pol);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // ------------------------------------------- MMA issuer
      const uint32_t idesc = tf32_idesc(TC_M, TC_N);
      int it = 0, g = 0;
      for (int tile = blockIdx.x; tile < ntiles && !*abort_v; tile += gridDim.x, it++) {
        const int acc = it & 1, use = it >> 1;
        if (use > 0 && !p_wait(&acc_empty[acc], (use - 1) & 1)) {
          *abort_v = 1;
          break;
        }
        const uint32_t d = tmem + static_cast<uint32_t>(acc * TC_N);
        bool ok = true;
        for (int kb = 0; kb < nkb; kb++, g++) {
          const int st = g % P_NST;
          if (!p_wait(&op_full[st], (g / P_NST) & 1)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t sp = smem_u32(base + st * stage_bytes);
          for (int k = 0; k < TC_KBLK / 8; k++) {
            const uint64_t koff = static_cast<uint64_t>((k * 32) >> 4);
            const uint64_t ad = sw128_desc(sp) + koff;
            const uint64_t bd = sw128_desc(sp + P_OPBLK_BYTES) + koff;
            uint32_t accum = (kb | k) ? 1u : 0u;
            if (split3) {  // small terms first: lo*hi, hi*lo, then hi*hi
              const uint64_t ald = sw128_desc(sp + 2 * P_OPBLK_BYTES) + koff;
              const uint64_t bld = sw128_desc(sp + 3 * P_OPBLK_BYTES) + koff;
              tf32_mma(d, ald, bd, idesc, accum);
              tf32_mma(d, ad, bld, idesc, 1u);
              accum = 1u;
            }
            tf32_mma(d, ad, bd, idesc, accum);
          }
          // the stage is free once these MMAs have read it
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                           smem_u32(&op_empty[st]))
                       : "memory");
        }
        if (!ok) {
          *abort_v = 1;
          break;
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(&acc_full[acc]))
                     : "memory");
      }
    }
  } else {  // ---------------------------------------------- epilogue (2-5)
    const int et = threadIdx.x - 64;      // 0..127
    const int quarter = warp & 3;         // TMEM lanes this warp may read
    const int row = quarter * 32 + lane;  // tile row
    int it = 0, cchunk = 0;
    int pend_slot = -1;  // slot whose TMA store may still be reading it (thread et == 0)
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, it++) {
      const int tm = tile % ntm, tn = tile / ntm;
      const int acc = it & 1;
      if (et == 0 && (*abort_v || !p_wait(&acc_full[acc], (it >> 1) & 1))) epi_abort = 1;
      asm volatile("bar.sync 1, 128;" ::: "memory");
      if (epi_abort) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int ch = 0; ch < TC_N / P_CCOLS; ch++, cchunk++) {
        const int slot = cchunk % ncs;
        if (et == 0 && !p_wait(&c_full[slot], (cchunk / ncs) & 1)) epi_abort = 1;
        asm volatile("bar.sync 1, 128;" ::: "memory");
        if (epi_abort) break;
        float* cs = reinterpret_cast<float*>(sC + slot * P_CHUNK_BYTES);  // [column][row]
        for (int c16 = 0; c16 < P_CCOLS; c16 += 16) {
          uint32_t r[16];
          const uint32_t taddr = tmem + (static_cast<uint32_t>(quarter * 32) << 16) +
                                 static_cast<uint32_t>(acc * TC_N + ch * P_CCOLS + c16);
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
              "[%16];"
              : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
              : "r"(taddr));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int q = 0; q < 16; q++) cs[(c16 + q) * TC_M + row] -= __uint_as_float(r[q]);
        }
        // generic-proxy writes -> visible to the TMA store
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        asm volatile("bar.sync 1, 128;" ::: "memory");
        if (et == 0) {
          p_tma_store_stream(&mapC, cs, tm * TC_M, tn * TC_N + ch * P_CCOLS, p_evict_first());
          asm volatile("cp.async.bulk.commit_group;" ::: "memory");
          // one store stays in flight: the previous chunk's slot is free
          // once its store has read it
          asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
          if (pend_slot >= 0) p_arrive(&c_empty[pend_slot]);
          pend_slot = slot;
          if (ch == TC_N / P_CCOLS - 1) p_arrive(&acc_empty[acc]);  // all 128 threads are past their loads
        }
      }
      if (epi_abort) break;
    }
    if (et == 0) {
      asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
      if (pend_slot >= 0) p_arrive(&c_empty[pend_slot]);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && (*abort_v || epi_abort)) atomicExch(err, 1);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256));
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no
// link-time dependency on the driver library).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// 2-D FP32 tensor map: inner extent `inner` (contiguous), `outer` rows
// `stride_bytes` apart, box box0 x box1.
void make_map(CUtensorMap* m, const void* ptr, long long inner, long long outer, long long stride_bytes, int box0,
              int box1, bool swizzle128) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) throw KdError(KD_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  cuuint64_t dims[2] = {static_cast<cuuint64_t>(inner), static_cast<cuuint64_t>(outer)};
  cuuint64_t strides[1] = {static_cast<cuuint64_t>(stride_bytes)};
  cuuint32_t box[2] = {static_cast<cuuint32_t>(box0), static_cast<cuuint32_t>(box1)};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(ptr), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw KdError(KD_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string(r) + ")");
}


int grid_for(long long n) {
  long long g = (n + 255) / 256;
  if (g > 152 * 8) g = 152 * 8;
  return static_cast<int>(g < 1 ? 1 : g);
}

}  // namespace

bool tf32_gemm_supported(int k) { return k > 0 && k <= TC_MAXK; }

bool tf32x3_gemm_possible(int k, const float* C, long long ldc, int m, int c_rows_writable) {
  const int kpad = ((k + TC_KBLK - 1) / TC_KBLK) * TC_KBLK;
  // the persistent pipeline's conditions (it streams k, so k may reach TC_MAXK_P)
  return k > 0 && kpad <= TC_MAXK_P && reinterpret_cast<uintptr_t>(C) % 16 == 0 && ldc % 4 == 0 &&
         (m + 3) / 4 * 4 <= c_rows_writable && encode_fn() != nullptr;
}

int tf32_update_max_clusters16() {
  static int maxc = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    if (cudaFuncSetAttribute(tf32_update_persistent, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
        cudaFuncSetAttribute(tf32_update_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(P_MAX_SMEM)) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    cudaLaunchConfig_t q = {};
    q.gridDim = dim3(16, 1, 1);
    q.blockDim = dim3(P_THREADS, 1, 1);
    q.dynamicSmemBytes = P_MAX_SMEM;
    cudaLaunchAttribute qa[1];
    qa[0].id = cudaLaunchAttributeClusterDimension;
    qa[0].val.clusterDim.x = 16;
    qa[0].val.clusterDim.y = 1;
    qa[0].val.clusterDim.z = 1;
    q.attrs = qa;
    q.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, tf32_update_persistent, &q) == cudaSuccess) maxc = n;
    cudaGetLastError();
  });
  return maxc;
}

void tf32_gemm_update(Context* ctx, int m, int n, int k, const float* A, long long lda, const float* B, long long ldb,
                      float* C, long long ldc, int c_rows_writable, int terms, int clusters, int max_ctas) {
  if (m <= 0 || n <= 0 || k <= 0) return;
  const bool split3 = (terms == 3);
  if (split3 && !tf32x3_gemm_possible(k, C, ldc, m, c_rows_writable))
    throw KdError(KD_ERR_UNSUPPORTED, "3xTF32 update needs k <= 192 and a 16-byte aligned C with ldc % 4 == 0");
  if (k > TC_MAXK && !split3) throw KdError(KD_ERR_ARG, "tcgen05 trailing update: panel width above 128");
  cudaStream_t s = ctx->stream();
  const int kpad = ((k + TC_KBLK - 1) / TC_KBLK) * TC_KBLK;
  const int mpad = ((m + TC_M - 1) / TC_M) * TC_M;
  const int npad = ((n + TC_N - 1) / TC_N) * TC_N;
  // hi parts first, lo parts (3xTF32) right after them
  size_t need_a = static_cast<size_t>(mpad) * kpad, need_b = static_cast<size_t>(npad) * kpad;
  // packed operands and the timeout flag live in the context's workspaces;
  // an update as clusters (the side stream's, beside the main stream's
  // updates of the next panel) packs into workspaces of its own
  const bool side = clusters != 0;
  float* at = static_cast<float*>(ctx->workspace(side ? Context::WS_TC_A2 : Context::WS_TC_A, 2 * need_a * sizeof(float)));
  float* bt = static_cast<float*>(ctx->workspace(side ? Context::WS_TC_B2 : Context::WS_TC_B, 2 * need_b * sizeof(float)));
  bool fresh = false;
  int* err = static_cast<int*>(ctx->workspace(Context::WS_TC_FLAG, sizeof(int), &fresh));
  if (fresh) cuda_check(cudaMemsetAsync(err, 0, sizeof(int), s), "memset err");
  float* at_lo = at + need_a;
  float* bt_lo = bt + need_b;
  // A is column-major m x k (contiguous along m); B is column-major k x n
  // (contiguous along k).
  pack_kmajor<<<grid_for(need_a), 256, 0, s>>>(A, lda, m, k, 1, at, split3 ? at_lo : nullptr, mpad, kpad);
  pack_kmajor<<<grid_for(need_b), 256, 0, s>>>(B, ldb, n, k, 0, bt, split3 ? bt_lo : nullptr, npad, kpad);
  ctx->launches += 2;
  const int nkb = kpad / TC_KBLK;
  // TMA clips the stored rows at 16-byte granularity: rows up to m rounded
  // to 4 may be written (with their unchanged values or zeros), so the
  // persistent path needs them to be scratch (c_rows_writable).
  const int m4 = (m + 3) / 4 * 4;
  if (reinterpret_cast<uintptr_t>(C) % 16 == 0 && ldc % 4 == 0 && m4 <= c_rows_writable && encode_fn()) {
    // persistent TMA pipeline
    CUtensorMap mA, mB, mAl, mBl, mC;
    make_map(&mA, at, kpad, mpad, static_cast<long long>(kpad) * 4, TC_KBLK, TC_M, true);
    make_map(&mB, bt, kpad, npad, static_cast<long long>(kpad) * 4, TC_KBLK, TC_N, true);
    make_map(&mAl, at_lo, kpad, mpad, static_cast<long long>(kpad) * 4, TC_KBLK, TC_M, true);
    make_map(&mBl, bt_lo, kpad, npad, static_cast<long long>(kpad) * 4, TC_KBLK, TC_N, true);
    make_map(&mC, C, m, n, ldc * 4, TC_M, P_CCOLS, false);
    static int nsm = 0;
    static std::once_flag pattr;
    std::call_once(pattr, [] {
      int dev = 0;
      cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
      cuda_check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev), "SM count");
      cuda_check(cudaFuncSetAttribute(tf32_update_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(P_MAX_SMEM)),
                 "cudaFuncSetAttribute(tf32 persistent)");
    });
    // shared memory: P_NST operand stages of one k-block each (x2 for the
    // lo parts), then as many C chunks as fit, up to P_CSLOTS
    const size_t ops = static_cast<size_t>(P_NST) * (split3 ? 4 : 2) * P_OPBLK_BYTES;
    int ncs = static_cast<int>((P_MAX_SMEM - 1024 - ops) / P_CHUNK_BYTES);
    if (ncs > P_CSLOTS) ncs = P_CSLOTS;
    const size_t psmem = 1024 + ops + static_cast<size_t>(ncs) * P_CHUNK_BYTES;
    if (psmem > P_MAX_SMEM) throw KdError(KD_ERR_UNSUPPORTED, "tcgen05 update: operands do not fit in shared memory");
    const int ntm = mpad / TC_M, ntiles = ntm * (npad / TC_N);
    const int maxc = clusters ? tf32_update_max_clusters16() : 0;
    if (maxc >= 2) {
      // 16-CTA clusters (the CTAs share nothing): one fewer than fit, or all
      int ncl = (ntiles + 15) / 16;
      const int cap = clusters == 2 ? maxc : maxc - 1;
      if (ncl > cap) ncl = cap;
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(16 * ncl, 1, 1);
      cfg.blockDim = dim3(P_THREADS, 1, 1);
      cfg.dynamicSmemBytes = psmem;
      cfg.stream = s;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = 16;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      cuda_check(cudaLaunchKernelEx(&cfg, tf32_update_persistent, mA, mB, mAl, mBl, mC, nkb, ntm, ntiles,
                                    split3 ? 1 : 0, ncs, err),
                 "tcgen05 trailing update (clusters)");
      ctx->launches += 1;
      return;
    }
    int cap = ctx->sms() < nsm ? ctx->sms() : nsm;
    if (max_ctas > 0 && max_ctas < cap) cap = max_ctas;
    const int grid = ntiles < cap ? ntiles : cap;
    tf32_update_persistent<<<grid, P_THREADS, psmem, s>>>(mA, mB, mAl, mBl, mC, nkb, ntm, ntiles, split3 ? 1 : 0, ncs,
                                                          err);
    ctx->launches += 1;
    cuda_check(cudaGetLastError(), "tcgen05 trailing update (persistent)");
    return;
  }
  // Each CTA holds 128 TMEM columns of the SM's 512: asking for at least
  // 56 KiB of shared memory keeps at most four CTAs on one SM, so an
  // allocation never has to wait for another CTA to finish.
  size_t smem = 1024 + static_cast<size_t>(2 * nkb) * 128 * 128;
  if (smem < TC_MIN_SMEM) smem = TC_MIN_SMEM;
  static std::once_flag attr;
  std::call_once(attr, [] {
    cuda_check(cudaFuncSetAttribute(tf32_update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    1024 + 2 * (TC_MAXK / TC_KBLK) * 128 * 128),
               "cudaFuncSetAttribute(tf32)");
  });
  dim3 grid(mpad / TC_M, npad / TC_N);
  tf32_update_kernel<<<grid, TC_THREADS, smem, s>>>(at, bt, kpad, C, ldc, m, n, err);
  ctx->launches += 1;
  cuda_check(cudaGetLastError(), "tcgen05 trailing update");
}

int tf32_gemm_error_flag(Context* ctx) {
  bool fresh = false;
  int* err = static_cast<int*>(ctx->workspace(Context::WS_TC_FLAG, sizeof(int), &fresh));
  if (fresh) {  // no update has run on this context yet
    cuda_check(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream()), "memset err");
    return 0;
  }
  int h = 0;
  cuda_check(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream()), "D2H err");
  cuda_check(cudaStreamSynchronize(ctx->stream()), "sync");
  if (h) cuda_check(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream()), "reset err");
  return h;
}

void gemm_update_f32(Context* ctx, cublasHandle_t blas, int m, int n, int k, const float* A, long long lda,
                     const float* B, long long ldb, float* C, long long ldc, bool tf32, int c_rows_writable,
                     int terms, int clusters, int max_ctas) {
  // work: the algorithmic HBM bytes (C read and written once, A and B read
  // once); the update is bound by the C stream
  ProfScope ps(ctx, Context::PROF_LU_GEMM, 8.0 * m * n + 4.0 * (static_cast<double>(m) + n) * k);
  if (tf32 && (tf32_gemm_supported(k) || (terms == 3 && tf32x3_gemm_possible(k, C, ldc, m, c_rows_writable)))) {
    if (terms == 3 && !tf32x3_gemm_possible(k, C, ldc, m, c_rows_writable)) terms = 1;
    tf32_gemm_update(ctx, m, n, k, A, lda, B, ldb, C, ldc, c_rows_writable, terms, clusters, max_ctas);
    return;
  }
  // plain FP32 product (the FP32-IR mode): library SGEMM
  const float one = 1.0f, mone = -1.0f;
  cublasStatus_t st = cublasGemmEx(blas, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &mone, A, CUDA_R_32F, static_cast<int>(lda),
                                   B, CUDA_R_32F, static_cast<int>(ldb), &one, C, CUDA_R_32F, static_cast<int>(ldc),
                                   CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
  if (st != CUBLAS_STATUS_SUCCESS) throw KdError(KD_ERR_CUDA, "cublasGemmEx (trailing update) failed");
  ctx->launches++;
}

}  // namespace kd
