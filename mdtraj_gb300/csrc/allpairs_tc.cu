// All-pairs and cross RMSD on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// P = X Y^T with each operand split into two BF16 planes (hi + lo), computed
// as hi.hi^T + hi.lo^T + lo.hi^T with FP32 accumulation in tensor memory (the
// lo.lo^T term is ~2^-18 relative and dropped).  One tile is a 128 x 240 block
// of P: 42 row frames (126 rows + 2 ignored) by 80 column frames.
//
// The tensor core's FP32 accumulator loses a fraction of an ulp per add in
// one direction; over the 384 accumulation steps of a 2,048-atom tile that
// biases msd by ~1e-4 nm^2.  The MMAs therefore accumulate only KFOLD k blocks
// (3 x 64 atoms, 36 steps; measured fastest of 2-4, max error 2.2e-5 nm on
// the 2,000-atom workload) into the partial buffer P in tensor memory, and
// CUDA-core warps fold P into FP32 registers with round-to-nearest adds (the
// promotion of partial sums used for low-precision tensor GEMMs).
//
// Persistent CTAs (one per SM), 448 threads:
//   warp 0       TMA producer: per 64-atom k block, four 2-D tensor copies
//                (A_hi, A_lo 128 x 64; B_hi, B_lo 240 x 64; 128-byte swizzle)
//                into a 2-stage shared-memory ring;
//   warp 1       allocates 512 TMEM columns -- P (columns 0-239) and the
//                result buffer R (256-495) -- and one lane issues the MMAs:
//                12 tcgen05.mma per k block (3 products x 4 k-steps of 16),
//                committing each stage's release and each fold unit's
//                completion to mbarriers;
//   warps 2..13  workers: warp w owns TMEM lanes 32*(w%4).. and 80 of the 240
//                columns.  For every fold unit of tile t they add P into 80
//                registers, release P, and then run one pass of the epilogue of
//                tile t-1, which waits in R: a pass stages a 48-column chunk of
//                R in shared memory (first pass of a chunk) and solves QCP in
//                FP32 (allpairs.cuh) for up to 384 of the chunk's 672 frame
//                pairs.  At the end of tile t (after finishing tile t-1's
//                passes) they store their registers into R.  So the epilogue
//                of one tile runs while the tensor cores work on the next.
// Every wait is bounded; the workers agree on a failure at every fold unit
// (barrier with an OR reduction) so that no named barrier can be left half
// entered; the CTA frees its tensor memory before exiting.
//
// Frames of at most 320 atoms (5 k blocks) use the DIRECT variant, 864
// threads: the MMAs of a tile accumulate all its k blocks in one of two
// tensor-memory buffers (no fold), alternating by tile; warps 2-5 stage the
// finished buffer into shared memory chunk by chunk, and warps 6-26 solve one
// frame pair each per chunk.  Stagers and solvers hand over through two
// mbarriers (chunk staged / chunk read by every solver), so a solver copies
// its 3x3 block to registers and goes on, and only the staging of the chunk
// after next waits for it.
#include <cuda.h>
#include <cuda_bf16.h>
#include <string.h>

#include <vector>

#include "allpairs.cuh"
#include "capi_internal.h"
#include "common.cuh"

namespace gb {
namespace {

constexpr int TILE_M = 128;             // rows of P per tile (tensor-core M)
constexpr int TILE_N = 240;             // columns of P per tile (tensor-core N)
constexpr int FR_M = 42;                // frames per tile row block (126 rows)
constexpr int FR_N = 80;                // frames per tile column block
constexpr int KBLK = 64;                // atoms per k block (128 B of BF16 = one swizzle row)
#ifndef GB_TC_KFOLD
#define GB_TC_KFOLD 3
#endif
constexpr int KFOLD = GB_TC_KFOLD;      // k blocks accumulated in P per fold
constexpr int NSTAGE = 2;
constexpr int A_BYTES = TILE_M * KBLK * 2;  // 16 KB
constexpr int B_BYTES = TILE_N * KBLK * 2;  // 30 KB
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
constexpr int EPI_COLS = 48;            // 16 frames per epilogue chunk
constexpr int EPI_LD = EPI_COLS + 1;
constexpr int EPI_BYTES = TILE_M * EPI_LD * 4;
constexpr int NCHUNK = TILE_N / EPI_COLS;       // 5 chunks per tile
constexpr int CHUNK_PAIRS = FR_M * 16;          // 672 frame pairs per chunk
constexpr int TMEM_COLS = 512;
constexpr uint32_t P_COL = 0;           // partial (fold) buffer
constexpr uint32_t R_COL = 256;         // result buffer of the tile awaiting its epilogue
constexpr int NGROUP = 3;               // column groups per TMEM lane slice
constexpr int GCOLS = TILE_N / NGROUP;  // 80 accumulator registers per thread
constexpr int NEPI = 4 * NGROUP;        // worker warps
constexpr int NEPI_THREADS = 32 * NEPI;
constexpr int NTHREADS = 64 + NEPI_THREADS;
constexpr int PASSES_PER_CHUNK = (CHUNK_PAIRS + NEPI_THREADS - 1) / NEPI_THREADS;  // 2
// DIRECT kernel (frames of at most DIRECT_MAX_KB k blocks, 320 atoms): no
// accumulators in registers, so a thread needs ~72 of them and 25 epilogue
// warps fit: 4 stagers (one per tensor-memory lane slice: three 16-column
// loads each per chunk) and 21 solvers, one thread per frame pair of a
// chunk, ~6 warps per scheduler to hide the epilogue's dependent FP32 chains.
// Stagers and solvers hand chunks over through two mbarriers (chunk staged;
// chunk read), so a solver that has copied its 3x3 block into registers
// never waits for a slower solver's QCP before the next chunk is staged.
constexpr int DIRECT_MAX_KB = 5;
constexpr int NSTAGER_D = 4;
constexpr int NEPI_D = (CHUNK_PAIRS + 31) / 32;          // 21 solver warps
constexpr int NEPI_D_THREADS = 32 * NEPI_D;             // 672
constexpr int NTHREADS_D = 64 + 32 * NSTAGER_D + NEPI_D_THREADS;  // 864
static_assert(NEPI_D_THREADS >= CHUNK_PAIRS, "one pair per solver thread per chunk");
__host__ __device__ constexpr int kernel_threads(bool direct) { return direct ? NTHREADS_D : NTHREADS; }
// Limit of one pipeline wait (a k block landing, a tile finishing, a chunk
// staged): far above any step of a healthy kernel, which takes microseconds.
constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;
static_assert(EPI_COLS == NGROUP * 16, "one 16-column TMEM load per worker warp per chunk");
static_assert(R_COL + TILE_N <= TMEM_COLS && P_COL + TILE_N <= R_COL, "TMEM layout");

// smem: [stages | epilogue staging | barriers | tmem address | cross column views]
constexpr int SMEM_STAGES = NSTAGE * STAGE_BYTES;
constexpr int SMEM_EPI = SMEM_STAGES;
constexpr int SMEM_BAR = SMEM_EPI + ((EPI_BYTES + 127) / 128) * 128;
constexpr int SMEM_COLV = SMEM_BAR + 128;
constexpr int SMEM_G = SMEM_COLV + FR_N * (int)sizeof(CrossCol);  // traces of the tile's frames as float
constexpr int SMEM_TOTAL = SMEM_G + (FR_M + FR_N) * 4 + 1024;        // + slack for 1024-byte alignment

struct TcArgs {
  const double* G;    // traces of the row frames
  const int2* tiles;  // (row block, column block)
  int64_t n_tiles;    // tile count, or an upper bound of it when n_tiles_dev is set
  const int64_t* n_tiles_dev;  // tile count written by an earlier kernel on the stream (cross calls)
  int64_t F;          // row frames (all-pairs: also the column frames)
  int32_t A;
  int32_t kpad;
  float* out;         // all-pairs output (F x F)
  PairRefine* rl;
  int* rc;
  int rcap;
  int* err;
  // cross RMSD only: column frames come from a query set
  const double* Gb;
  const gbrmsd_cross_request_t* reqs;
  const int32_t* colreq;
  int64_t n_b;
};

// ---- PTX wrappers ----------------------------------------------------------

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int32_t x, int32_t y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(smem_addr(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void tc_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst_smem)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int t = 0; t < 16; ++t) v[t] = __uint_as_float(r[t]);
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void named_bar(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, rows of
// 128 bytes, 8-row core groups 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);  // start address
  d |= (uint64_t)1 << 16;                  // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;        // stride byte offset
  d |= (uint64_t)1 << 46;                  // descriptor version for tcgen05
  d |= (uint64_t)2 << 61;                  // swizzle: 128 B
  return d;
}

// Instruction descriptor: kind::f16, BF16 x BF16 -> F32, both K-major, M x N.
__host__ __device__ constexpr uint32_t make_idesc(int m, int n) {
  return (1u << 4)                       // D format F32
         | (1u << 7)                     // A format BF16
         | (1u << 10)                    // B format BF16
         | ((uint32_t)(n >> 3) << 17)    // N / 8
         | ((uint32_t)(m >> 4) << 24);   // M / 16
}

__device__ __forceinline__ bool wait_bar(uint64_t* bar, uint32_t parity, int* err) {
  return mbar_wait_sleep(bar, parity, err, WAIT_LIMIT_NS);
}

__device__ __forceinline__ void tc_st16(uint32_t taddr, const float (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16};" ::"r"(taddr),
      "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
      "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
      "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])),
      "r"(__float_as_uint(v[11])), "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])),
      "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15]))
      : "memory");
}
__device__ __forceinline__ void tc_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Named barrier that also ORs a flag over its n threads: every thread gets the
// same answer, so a decision taken on it cannot split the group.
__device__ __forceinline__ bool named_bar_or(int id, int n, bool v) {
  int r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.b32 q, %1, 0;\n\t"
      "bar.red.or.pred p, %2, %3, q;\n\t"
      "selp.b32 %0, 1, 0, p;\n\t}"
      : "=r"(r)
      : "r"((int)v), "r"(id), "r"(n)
      : "memory");
  return r != 0;
}

// DIRECT: each tile accumulates all its k blocks in one of two tensor-memory
// buffers (columns 0-239 and 256-495), alternating by tile, with no fold into
// registers; the workers' epilogue reads the finished buffer while the MMAs
// fill the other.  The accumulator then takes at most 5 x 12 = 60 steps,
// against the 36 of a fold unit.
template <bool CROSS, bool DIRECT>
__global__ void __launch_bounds__(kernel_threads(DIRECT), 1) allpairs_tc_kernel(const __grid_constant__ CUtensorMap map_hi_a,
                                                                  const __grid_constant__ CUtensorMap map_lo_a,
                                                                  const __grid_constant__ CUtensorMap map_hi_b,
                                                                  const __grid_constant__ CUtensorMap map_lo_b,
                                                                  const TcArgs args) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte aligned for the 128-byte swizzle; an offset from the shared
  // array (not an integer cast) keeps every access below a shared-memory one
  unsigned char* smem = smem_raw + ((1024u - (smem_addr(smem_raw) & 1023u)) & 1023u);
  float* sD = reinterpret_cast<float*>(smem + SMEM_EPI);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + SMEM_BAR);
  uint64_t* full = bars;                  // [NSTAGE] operands landed
  uint64_t* empty = bars + NSTAGE;        // [NSTAGE] operands consumed by the MMAs
  uint64_t* pfull = bars + 2 * NSTAGE;    // [2] P holds a finished fold unit (DIRECT: buffer b holds a tile)
  uint64_t* pempty = pfull + 2;           // [2] P folded by all worker warps (DIRECT: buffer b read)
  uint64_t* sfull = pempty + 2;           // DIRECT: a chunk is staged in shared memory
  uint64_t* sfree = sfull + 1;            // DIRECT: every solver has read the staged chunk
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sfree + 1);
  volatile int* fail_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  CrossCol* colv = reinterpret_cast<CrossCol*>(smem + SMEM_COLV);
  float* sGa = reinterpret_cast<float*>(smem + SMEM_G);  // [FR_M] row frames of the pending tile
  float* sGb = sGa + FR_M;                               // [FR_N] column frames

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&pfull[b], 1);
      mbar_init(&pempty[b], DIRECT ? NSTAGER_D : NEPI);
    }
    mbar_init(sfull, 32 * NSTAGER_D);
    mbar_init(sfree, NEPI_D_THREADS);
    *fail_flag = 0;
    fence_mbar_init();
  }
  if (warp == 1) {
    tc_alloc(tmem_slot, TMEM_COLS);
    tc_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  const int64_t n_tiles = args.n_tiles_dev ? *args.n_tiles_dev : args.n_tiles;
  const int nkb = args.kpad / KBLK;
  const int nunit = (nkb + KFOLD - 1) / KFOLD;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
        const int2 tl = args.tiles[t];
        const int32_t row_a = tl.x * (3 * FR_M), row_b = tl.y * (3 * FR_N);
        for (int kb = 0; kb < nkb; ++kb, ++it) {
          const int s = it % NSTAGE;
          const uint32_t use = it / NSTAGE;
          if ((use > 0 && !wait_bar(&empty[s], (use - 1) & 1, args.err)) || *fail_flag) {
            *fail_flag = 1;
            ok = false;
            break;
          }
          unsigned char* st = smem + s * STAGE_BYTES;
          mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
          tma_load_2d(st, &map_hi_a, kb * KBLK, row_a, &full[s]);
          tma_load_2d(st + A_BYTES, &map_lo_a, kb * KBLK, row_a, &full[s]);
          tma_load_2d(st + 2 * A_BYTES, &map_hi_b, kb * KBLK, row_b, &full[s]);
          tma_load_2d(st + 2 * A_BYTES + B_BYTES, &map_lo_b, kb * KBLK, row_b, &full[s]);
        }
      }
      // no copy may still be landing when the CTA exits
      for (uint32_t k = (it > NSTAGE ? it - NSTAGE : 0); k < it; ++k)
        if (!wait_bar(&full[k % NSTAGE], (k / NSTAGE) & 1, args.err)) break;
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0 && DIRECT) {
      constexpr uint32_t idesc = make_idesc(TILE_M, TILE_N);
      uint32_t it = 0, k = 0;  // k blocks issued, tiles committed
      bool ok = true;
      for (int64_t t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
        const uint32_t buf = k & 1;
        if (k >= 2 && (!wait_bar(&pempty[buf], ((k - 2) >> 1) & 1, args.err) || *fail_flag)) {
          *fail_flag = 1;
          ok = false;
          break;
        }
        const uint32_t d_tmem = tmem_base + (buf ? R_COL : P_COL);
        for (int kb = 0; kb < nkb; ++kb, ++it) {
          const int s = it % NSTAGE;
          if (!wait_bar(&full[s], (it / NSTAGE) & 1, args.err)) {
            *fail_flag = 1;
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t st = smem_addr(smem + s * STAGE_BYTES);
          const uint32_t a_hi = st, a_lo = st + A_BYTES, b_hi = st + 2 * A_BYTES, b_lo = st + 2 * A_BYTES + B_BYTES;
#pragma unroll
          for (int ks = 0; ks < KBLK / 16; ++ks) {
            const uint32_t koff = ks * 32;
            tc_mma(d_tmem, smem_desc_sw128(a_hi + koff), smem_desc_sw128(b_hi + koff), idesc,
                   (kb == 0 && ks == 0) ? 0u : 1u);
            tc_mma(d_tmem, smem_desc_sw128(a_hi + koff), smem_desc_sw128(b_lo + koff), idesc, 1u);
            tc_mma(d_tmem, smem_desc_sw128(a_lo + koff), smem_desc_sw128(b_hi + koff), idesc, 1u);
          }
          tc_commit(&empty[s]);
        }
        if (!ok) break;
        tc_commit(&pfull[buf]);  // the tile is complete in buffer buf
        ++k;
      }
      if (k > 0) wait_bar(&pfull[(k - 1) & 1], ((k - 1) >> 1) & 1, args.err);  // no MMA left in flight
    } else if (lane == 0) {
      constexpr uint32_t idesc = make_idesc(TILE_M, TILE_N);
      const uint32_t d_tmem = tmem_base + P_COL;
      uint32_t it = 0, unit = 0;  // k blocks issued, fold units committed
      bool ok = true;
      for (int64_t t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
        for (int kb = 0; kb < nkb; ++kb, ++it) {
          const bool first = (kb % KFOLD) == 0;
          if (first && unit > 0 && (!wait_bar(pempty, (unit - 1) & 1, args.err) || *fail_flag)) {
            *fail_flag = 1;
            ok = false;
            break;
          }
          const int s = it % NSTAGE;
          if (!wait_bar(&full[s], (it / NSTAGE) & 1, args.err)) {
            *fail_flag = 1;
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t st = smem_addr(smem + s * STAGE_BYTES);
          const uint32_t a_hi = st, a_lo = st + A_BYTES, b_hi = st + 2 * A_BYTES, b_lo = st + 2 * A_BYTES + B_BYTES;
#pragma unroll
          for (int ks = 0; ks < KBLK / 16; ++ks) {
            const uint32_t koff = ks * 32;  // 16 BF16 = 32 bytes inside the 128-byte swizzle row
            tc_mma(d_tmem, smem_desc_sw128(a_hi + koff), smem_desc_sw128(b_hi + koff), idesc,
                   (first && ks == 0) ? 0u : 1u);
            tc_mma(d_tmem, smem_desc_sw128(a_hi + koff), smem_desc_sw128(b_lo + koff), idesc, 1u);
            tc_mma(d_tmem, smem_desc_sw128(a_lo + koff), smem_desc_sw128(b_hi + koff), idesc, 1u);
          }
          tc_commit(&empty[s]);  // operand stage reusable once these MMAs have read it
          if ((kb % KFOLD) == KFOLD - 1 || kb == nkb - 1) {
            tc_commit(pfull);    // fold unit complete in P
            ++unit;
          }
        }
      }
      if (unit > 0) wait_bar(pfull, (unit - 1) & 1, args.err);  // no MMA left in flight
    }
  } else {
    // ---------------- DIRECT: stager and solver warps ----------------
    if constexpr (DIRECT) {
      const float inv_n = 1.0f / (float)args.A;
      bool failed = false;
      uint32_t k = 0, g = 0;  // tiles, chunks of this CTA
      if (warp < 2 + NSTAGER_D) {
        // stager: tile k's buffer into shared memory, chunk by chunk
        const int slice = warp & 3;
        const int sid = (warp - 2) * 32 + lane;  // 0 .. 127
        const uint32_t lane_off = (uint32_t)(slice * 32) << 16;
        float* dst = sD + (slice * 32 + lane) * EPI_LD;
        for (int64_t t = blockIdx.x; t < n_tiles && !failed; t += gridDim.x, ++k) {
          const uint32_t buf = k & 1;
          if (!wait_bar(&pfull[buf], (k >> 1) & 1, args.err) || *fail_flag) {
            failed = true;
            break;
          }
          tc_fence_after();
          const int2 tl = args.tiles[t];
          const int64_t pi0 = (int64_t)tl.x * FR_M, pj0 = (int64_t)tl.y * FR_N;
          const uint32_t tcol = buf ? R_COL : P_COL;
          for (int ch = 0; ch < NCHUNK; ++ch, ++g) {
            if (g > 0 && (!wait_bar(sfree, (g - 1) & 1, args.err) || *fail_flag)) {
              failed = true;
              break;
            }
            if (ch == 0) {
              // per tile: the request of each column frame, and the frames'
              // traces rounded to float once (not per pair on the FP64 pipe)
              if (CROSS && sid < FR_N) colv[sid] = cross_col(args.reqs, args.colreq, pj0 + sid, args.n_b);
              if (sid < FR_M) sGa[sid] = pi0 + sid < args.F ? (float)args.G[pi0 + sid] : 0.f;
              if (sid < FR_N) {
                const int64_t j = pj0 + sid;
                sGb[sid] = CROSS ? (j < args.n_b ? (float)args.Gb[j] : 0.f) : (j < args.F ? (float)args.G[j] : 0.f);
              }
            }
#pragma unroll
            for (int q = 0; q < NGROUP; ++q) {
              float v[16];
              tc_ld16(tmem_base + tcol + (uint32_t)(ch * EPI_COLS + q * 16) + lane_off, v);
              tc_wait_ld();
#pragma unroll
              for (int c = 0; c < 16; ++c) dst[q * 16 + c] = v[c];
            }
            if (ch == NCHUNK - 1) {  // this warp's last read of the buffer
              tc_fence_before();
              __syncwarp();
              if (lane == 0) mbar_arrive(&pempty[buf]);
            }
            mbar_arrive(sfull);  // every stager thread: its stores are released to the solvers
          }
        }
      } else {
        // solver: one frame pair of every chunk
        const int p = (warp - 2 - NSTAGER_D) * 32 + lane;  // 0 .. 671
        int li, lj;
        if (CROSS) {
          // consecutive threads take consecutive row frames of one column
          // frame: contiguous in the request's output row
          lj = p / FR_M;
          li = p - lj * FR_M;
        } else {
          li = p >> 4;
          lj = p & 15;
        }
        for (int64_t t = blockIdx.x; t < n_tiles && !failed; t += gridDim.x, ++k) {
          const int2 tl = args.tiles[t];
          const int64_t i = (int64_t)tl.x * FR_M + li;
          for (int ch = 0; ch < NCHUNK; ++ch, ++g) {
            if (!wait_bar(sfull, g & 1, args.err) || *fail_flag) {
              failed = true;
              break;
            }
            float m[9];
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
              for (int d = 0; d < 3; ++d) m[3 * c + d] = sD[(3 * li + c) * EPI_LD + 3 * lj + d];
            const float ga = sGa[li], gb = sGb[ch * 16 + lj];
            const int64_t j = (int64_t)tl.y * FR_N + ch * 16 + lj;
            CrossCol cv;
            if (CROSS) cv = colv[ch * 16 + lj];
            mbar_arrive(sfree);  // this thread's reads of the chunk are done
            if (CROSS) {
              if (cv.row != nullptr && i >= cv.db0 && i < cv.db1 && i < args.F)
                cross_pair(i, j, m, ga, gb, inv_n, cv.row + (i - cv.db0), args.rl, args.rc, args.rcap, args.err);
            } else if (i < args.F && j < args.F && i <= j) {
              pair_epilogue_g(i, j, m, ga, gb, inv_n, args.F, args.out, args.rl, args.rc, args.rcap, args.err);
            }
          }
        }
      }
      if (failed) *fail_flag = 1;
    } else {
    // ---------------- worker warps (fold + interleaved epilogue) ----------------
    const int ew = warp - 2;              // 0 .. NEPI-1
    const int slice = warp & 3;           // TMEM lanes [32*slice, 32*slice + 32)
    const int grp = ew >> 2;              // column group: columns [80*grp, 80*grp + 80)
    const int row = slice * 32 + lane;    // accumulator row of this thread
    const int etid = ew * 32 + lane;      // 0 .. worker threads - 1
    constexpr int WT = NEPI_THREADS;                 // worker threads
    constexpr int ppc = PASSES_PER_CHUNK;            // passes per chunk
    constexpr int passes = NCHUNK * ppc;             // per tile (10)
    const float inv_n = 1.0f / (float)args.A;
    const uint32_t lane_off = (uint32_t)(slice * 32) << 16;
    bool pend = false;   // a tile waits in R for its epilogue
    int pass = 0;        // its next pass
    int64_t pi0 = 0, pj0 = 0;

    // One epilogue pass of the pending tile: the first pass of a chunk stages
    // the 48-column chunk from R into shared memory (one 16-column load per
    // warp), then every thread takes at most one of the chunk's 672 frame
    // pairs.
    auto do_pass = [&]() {
      const int ch = pass / ppc, sub = pass % ppc;
      if (sub == 0) {
        if (ch == 0) {
          // per tile: the request of each column frame, and the frames'
          // traces rounded to float once (not per pair on the FP64 pipe)
          if (CROSS && etid < FR_N) colv[etid] = cross_col(args.reqs, args.colreq, pj0 + etid, args.n_b);
          if (etid < FR_M) sGa[etid] = pi0 + etid < args.F ? (float)args.G[pi0 + etid] : 0.f;
          if (etid < FR_N) {
            const int64_t j = pj0 + etid;
            sGb[etid] = CROSS ? (j < args.n_b ? (float)args.Gb[j] : 0.f) : (j < args.F ? (float)args.G[j] : 0.f);
          }
        }
        float v[16];
        tc_ld16(tmem_base + R_COL + (uint32_t)(ch * EPI_COLS + grp * 16) + lane_off, v);
        tc_wait_ld();
        float* dst = sD + row * EPI_LD + grp * 16;
#pragma unroll
        for (int q = 0; q < 16; ++q) dst[q] = v[q];
        named_bar(1, WT);
      }
      const int p = sub * WT + etid;
      if (p < CHUNK_PAIRS) {
        if (CROSS) {
          // consecutive threads take consecutive row frames of one column frame:
          // contiguous in the request's output row
          const int lj = p / FR_M, li = p - lj * FR_M;
          const int64_t i = pi0 + li;
          const CrossCol cv = colv[ch * 16 + lj];
          if (cv.row != nullptr && i >= cv.db0 && i < cv.db1 && i < args.F) {
            float m[9];
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
              for (int d = 0; d < 3; ++d) m[3 * c + d] = sD[(3 * li + c) * EPI_LD + 3 * lj + d];
            const int64_t j = pj0 + ch * 16 + lj;
            cross_pair(i, j, m, sGa[li], sGb[ch * 16 + lj], inv_n, cv.row + (i - cv.db0), args.rl, args.rc,
                       args.rcap, args.err);
          }
        } else {
          const int li = p >> 4, lj = p & 15;
          const int64_t i = pi0 + li, j = pj0 + ch * 16 + lj;
          if (i < args.F && j < args.F && i <= j) {
            float m[9];
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
              for (int d = 0; d < 3; ++d) m[3 * c + d] = sD[(3 * li + c) * EPI_LD + 3 * lj + d];
            pair_epilogue_g(i, j, m, sGa[li], sGb[ch * 16 + lj], inv_n, args.F, args.out, args.rl, args.rc,
                            args.rcap, args.err);
          }
        }
      }
      if (sub == ppc - 1) {
        tc_fence_before();
        named_bar(1, WT);  // chunk (and, after the last, R) no longer read
        tc_fence_after();
      }
      if (++pass == passes) pend = false;
    };

    uint32_t unit = 0;
    bool failed = false;
    const int ppu = (passes + nunit - 1) / nunit;  // epilogue passes after each fold
    for (int64_t t = blockIdx.x; t < n_tiles && !failed; t += gridDim.x) {
      float acc[GCOLS];
#pragma unroll
      for (int q = 0; q < GCOLS; ++q) acc[q] = 0.f;
      for (int u = 0; u < nunit; ++u, ++unit) {
        const bool ok = __all_sync(FULL_MASK, wait_bar(pfull, unit & 1, args.err) && !*fail_flag);
        if (named_bar_or(2, NEPI_THREADS, !ok)) {  // one answer for all worker warps
          failed = true;
          break;
        }
        tc_fence_after();
        const uint32_t taddr = tmem_base + P_COL + (uint32_t)(grp * GCOLS) + lane_off;
#pragma unroll
        for (int c0 = 0; c0 < GCOLS; c0 += 16) {
          float v[16];
          tc_ld16(taddr + c0, v);
          tc_wait_ld();
#pragma unroll
          for (int q = 0; q < 16; ++q) acc[c0 + q] += v[q];
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(pempty);
        for (int r = 0; r < ppu && pend; ++r) do_pass();
      }
      if (failed) break;
      while (pend) do_pass();  // R must be free before this tile goes in
      {
        const uint32_t taddr = tmem_base + R_COL + (uint32_t)(grp * GCOLS) + lane_off;
#pragma unroll
        for (int c0 = 0; c0 < GCOLS; c0 += 16) {
          float v[16];
#pragma unroll
          for (int q = 0; q < 16; ++q) v[q] = acc[c0 + q];
          tc_st16(taddr + c0, v);
        }
        tc_wait_st();
      }
      tc_fence_before();
      named_bar(1, NEPI_THREADS);  // R complete for every worker warp
      tc_fence_after();
      const int2 tl = args.tiles[t];
      pi0 = (int64_t)tl.x * FR_M;
      pj0 = (int64_t)tl.y * FR_N;
      pend = true;
      pass = 0;
    }
    if (failed) *fail_flag = 1;
    else
      while (pend) do_pass();
    }  // fold kernel
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tc_dealloc(tmem_base, TMEM_COLS);
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn lookup_encode_tiled() {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    return nullptr;
  return reinterpret_cast<EncodeTiledFn>(p);
}

int encode_plane(CUtensorMap* tm, const void* base, int64_t rows, int32_t kpad, int box_rows) {
  // looked up once per process (a function-local static is initialised
  // exactly once even when host threads call concurrently)
  static const EncodeTiledFn fn = lookup_encode_tiled();
  if (!fn) return set_error(GBRMSD_E_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
  const cuuint64_t dims[2] = {(cuuint64_t)kpad, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)kpad * 2};
  const cuuint32_t box[2] = {KBLK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(GBRMSD_E_INVALID, "cuTensorMapEncodeTiled (bf16 plane) failed: %d", (int)r);
  return GBRMSD_OK;
}

// Tile list: groups of 8 row blocks, column-major inside a group, so tiles
// that run concurrently share column blocks (and row blocks) in L2.
std::vector<int2> make_tiles(int64_t F) {
  const int64_t nbr = (F + FR_M - 1) / FR_M, nbc = (F + FR_N - 1) / FR_N;
  std::vector<int2> tiles;
  const int64_t grp = 8;
  for (int64_t g0 = 0; g0 < nbr; g0 += grp) {
    const int64_t g1 = g0 + grp < nbr ? g0 + grp : nbr;
    for (int64_t cb = 0; cb < nbc; ++cb)
      for (int64_t rb = g0; rb < g1; ++rb) {
        // needed iff some pair (i, j) of the tile has i <= j
        if (cb * FR_N + FR_N - 1 >= rb * FR_M) tiles.push_back(make_int2((int)rb, (int)cb));
      }
  }
  return tiles;
}

}  // namespace

int launch_allpairs_tc(const __nv_bfloat16* Xhi, const __nv_bfloat16* Xlo, const double* G, int64_t F, int32_t A,
                       int32_t kpad, float* out, PairRefine* rl, int* rc, int rcap, int* err, cudaStream_t st) {
  if (kpad % KBLK) return set_error(GBRMSD_E_INVALID, "allpairs_tc: k padding must be a multiple of 64");
  if (max_dyn_smem() < SMEM_TOTAL) return set_error(GBRMSD_E_UNSUPPORTED, "allpairs_tc: not enough shared memory");
  const int64_t rows = 3 * F;
  alignas(64) CUtensorMap mha, mla, mhb, mlb;
  memset(&mha, 0, sizeof(mha));
  memset(&mla, 0, sizeof(mla));
  memset(&mhb, 0, sizeof(mhb));
  memset(&mlb, 0, sizeof(mlb));
  int rc0 = encode_plane(&mha, Xhi, rows, kpad, TILE_M);
  if (!rc0) rc0 = encode_plane(&mla, Xlo, rows, kpad, TILE_M);
  if (!rc0) rc0 = encode_plane(&mhb, Xhi, rows, kpad, TILE_N);
  if (!rc0) rc0 = encode_plane(&mlb, Xlo, rows, kpad, TILE_N);
  if (rc0) return rc0;
  const std::vector<int2> tiles = make_tiles(F);
  // tile list lives right after the refinement list in the caller's workspace
  int2* dtiles = reinterpret_cast<int2*>(reinterpret_cast<unsigned char*>(rl) + align_up((size_t)rcap * sizeof(PairRefine), 256));
  GB_CUDA_TRY(cudaMemcpyAsync(dtiles, tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice, st),
              "copy tile list");
  TcArgs a;
  a.G = G;
  a.tiles = dtiles;
  a.n_tiles = (int64_t)tiles.size();
  a.n_tiles_dev = nullptr;
  a.F = F;
  a.A = A;
  a.kpad = kpad;
  a.out = out;
  a.rl = rl;
  a.rc = rc;
  a.rcap = rcap;
  a.err = err;
  a.Gb = nullptr;
  a.reqs = nullptr;
  a.colreq = nullptr;
  a.n_b = 0;
  const int64_t grid = a.n_tiles < sm_count() ? a.n_tiles : sm_count();
  if (kpad / KBLK <= DIRECT_MAX_KB) {
    GB_CUDA_TRY(cudaFuncSetAttribute(allpairs_tc_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     SMEM_TOTAL),
                "cudaFuncSetAttribute(allpairs_tc_kernel)");
    allpairs_tc_kernel<false, true><<<(unsigned)grid, NTHREADS_D, SMEM_TOTAL, st>>>(mha, mla, mhb, mlb, a);
  } else {
    GB_CUDA_TRY(cudaFuncSetAttribute(allpairs_tc_kernel<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     SMEM_TOTAL),
                "cudaFuncSetAttribute(allpairs_tc_kernel)");
    allpairs_tc_kernel<false, false><<<(unsigned)grid, NTHREADS, SMEM_TOTAL, st>>>(mha, mla, mhb, mlb, a);
  }
  GB_CUDA_TRY(cudaGetLastError(), "launch allpairs_tc_kernel");
  // (a pageable host->device cudaMemcpyAsync returns once the source has been
  // staged, so the host tile list may go out of scope here)
  return GBRMSD_OK;
}

int launch_cross_tc(const __nv_bfloat16* Ahi, const __nv_bfloat16* Alo, const double* Ga, int64_t n_a, int64_t cap_a,
                    const __nv_bfloat16* Bhi, const __nv_bfloat16* Blo, const double* Gb, int64_t cap_b, int32_t A,
                    int32_t kpad, const gbrmsd_cross_request_t* reqs, const int32_t* colreq, const int2* tiles,
                    int64_t max_tiles, const int64_t* n_tiles_dev, PairRefine* rl, int* rc, int rcap, int* err,
                    cudaStream_t st) {
  if (kpad % KBLK) return set_error(GBRMSD_E_INVALID, "cross_tc: k padding must be a multiple of 64");
  if (max_dyn_smem() < SMEM_TOTAL) return set_error(GBRMSD_E_UNSUPPORTED, "cross_tc: not enough shared memory");
  if (max_tiles == 0) return GBRMSD_OK;
  const int64_t n_tiles = max_tiles;
  alignas(64) CUtensorMap mha, mla, mhb, mlb;
  memset(&mha, 0, sizeof(mha));
  memset(&mla, 0, sizeof(mla));
  memset(&mhb, 0, sizeof(mhb));
  memset(&mlb, 0, sizeof(mlb));
  int rc0 = encode_plane(&mha, Ahi, 3 * cap_a, kpad, TILE_M);
  if (!rc0) rc0 = encode_plane(&mla, Alo, 3 * cap_a, kpad, TILE_M);
  if (!rc0) rc0 = encode_plane(&mhb, Bhi, 3 * cap_b, kpad, TILE_N);
  if (!rc0) rc0 = encode_plane(&mlb, Blo, 3 * cap_b, kpad, TILE_N);
  if (rc0) return rc0;
  TcArgs a;
  a.G = Ga;
  a.tiles = tiles;
  a.n_tiles = n_tiles;
  a.n_tiles_dev = n_tiles_dev;
  a.F = n_a;
  a.A = A;
  a.kpad = kpad;
  a.out = nullptr;
  a.rl = rl;
  a.rc = rc;
  a.rcap = rcap;
  a.err = err;
  a.Gb = Gb;
  a.reqs = reqs;
  a.colreq = colreq;
  a.n_b = cap_b;
  const int64_t grid = n_tiles < sm_count() ? n_tiles : sm_count();
  if (kpad / KBLK <= DIRECT_MAX_KB) {
    GB_CUDA_TRY(cudaFuncSetAttribute(allpairs_tc_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     SMEM_TOTAL),
                "cudaFuncSetAttribute(cross_tc_kernel)");
    allpairs_tc_kernel<true, true><<<(unsigned)grid, NTHREADS_D, SMEM_TOTAL, st>>>(mha, mla, mhb, mlb, a);
  } else {
    GB_CUDA_TRY(cudaFuncSetAttribute(allpairs_tc_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     SMEM_TOTAL),
                "cudaFuncSetAttribute(cross_tc_kernel)");
    allpairs_tc_kernel<true, false><<<(unsigned)grid, NTHREADS, SMEM_TOTAL, st>>>(mha, mla, mhb, mlb, a);
  }
  GB_CUDA_TRY(cudaGetLastError(), "launch cross_tc_kernel");
  return GBRMSD_OK;
}

int cross_tc_block_frames(int* rows, int* cols) {
  *rows = FR_M;
  *cols = FR_N;
  return GBRMSD_OK;
}

size_t allpairs_tc_tiles_bytes(int64_t F) {
  const int64_t nbr = (F + FR_M - 1) / FR_M, nbc = (F + FR_N - 1) / FR_N;
  return align_up((size_t)(nbr * nbc) * sizeof(int2), 256);
}

}  // namespace gb
