// Tensor-core form of the field's six GEMMs (GB300, sm_103a): tcgen05.mma (kind::f16, bf16 operands, float32
// accumulation in tensor memory), operands staged by TMA (cp.async.bulk.tensor, 128-byte swizzle) through an
// mbarrier pipeline, one elected thread issuing the MMAs, four warps reading the accumulator back (tcgen05.ld) into
// fused epilogues, with the accumulation promoted to float32 registers after every k-block (below). Operands are
// float32 values split into bf16 terms, a = a0 + a1 + a2 (each term the bf16 rounding of what the previous ones
// leave), stored as three planes; a product is a list of (A term, B term) pairs over the same K, all issued on the
// same staged k-block (each term's tile is loaded once per k-block) into one accumulator:
//   bf16x3: (1,0) (0,1) (0,0)                          ~1e-5 of the max
//   bf16x6: (2,0) (1,1) (0,2) (1,0) (0,1) (0,0)        ~2e-7 of the max (float32-level)
// f16x3 instead keeps two float16 terms per operand, data chunks scaled by powers of two (below), 3 products.
// tf32x3 keeps two tf32 terms per operand as float32 planes (kind::tf32 MMAs: a 128-byte row is 32 of K), 3 products
// as bf16x3's.
// Tiles are 128 rows x BN columns: BN = 64 when a launch has one GEMM (twice the blocks), 128 when it has two.
// Folded transforms (f16x3, grids of multiples of 256; field.cuh): the forward ones as two half-size GEMMs per launch
// (64-column tiles; the first with EPI_FOLD, 64-row B tiles and their mirrors), the inverse ones as half-height
// tiles that also write their mirror rows (EPI_MSPLIT, EPI_MPLAIN).
// Shapes: M, N multiples of 128, K a multiple of 64 (force grids of 128 .. 4096 bins per side).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "field.cuh"
#include "gp103.cuh"

namespace gp103 {

constexpr int TC_BM = 128, TC_BK = 64;                           // TC_BK: 16-bit elements of K per k-block
constexpr int TC_A_TILE = TC_BM * TC_BK * 2;                     // 16 KB per A term tile (128-byte rows, any mode)
constexpr int TC_STAGE_SPACE = 216 * 1024;                       // room for the stages
constexpr int TC_MAX_STAGES = 4;
constexpr int TC_SMEM = TC_STAGE_SPACE + 1024 + 256;
constexpr long long TC_DRAIN_NS = 2000000000LL;                 // limit of the waits for work already in flight
constexpr int EPI_BOX = 128 * 128;                               // an epilogue box: 128 rows x 128 bytes

struct TcProblem {
    int M, N, K;
    int epi;
    int M_out, m_out;            // the outputs (terms, float32 plane, exponents) have M_out rows; this problem's start
                                 // at row m_out (two problems of one launch can fill one output)
    int msign;                   // MSPLIT / MPLAIN: +1 for a cosine row operand (mirror row E - O), -1 for a sine one
    __nv_bfloat16* o_terms;      // EPI_SPLIT: [3][M][N]; EPI_WEIGHT2: [3][M][N] (Kx), o2: Ky
    __nv_bfloat16* o2_terms;
    float* out_f32;              // EPI_PLAIN: [M][N]
    const float4* wrow;          // EPI_WEIGHT2: per row p (kx^2, s kx / bin_x, w_p, 0)
    const float4* wcol;          //              per column q (ky^2, s ky / bin_x, w_q, 0)
    // f16x3: exponents of the B operand's chunks, [K / 64][N] (B row n, k-block kb: its terms hold b * 2^e), and of
    // the outputs' chunks, [N / 64][M] (written by the epilogue: the next GEMM reads the output as its B operand)
    const signed char* b_exp;
    signed char* o_exp;
    signed char* o2_exp;
};

// A stage holds the k-block (64 of K) of every term of A and of B that the products read: na A tiles, then nb B
// tiles. Each of the nprod products (ia, ib) is four MMAs over that k-block, all into one accumulator, in the order
// given (smallest first, so the truncating accumulation adds small terms while the sum is small).
struct TcArgs {
    TcProblem p[2];
    int stages;
    int* err;
    long long wait_ns;           // limit of one wait (GP103_OPT_WAIT_MS)
    int stall;                   // GP103_OPT_TEST_STALL_FIELD: the producer issues no load (every wait runs out)
    int early;                   // bit 0: A of the first stages loaded before the dependency wait; bit 1: the next
                                 // kernel may launch once this block's accumulation is done
};

// The products of a mode, smallest first: bf16x6 (X6 = 1) has 3 terms per operand and 6 products, bf16x3 2 and 3.
__device__ __forceinline__ constexpr int prod_a(int x6, int q) {
    return x6 ? (q == 0 ? 2 : q == 1 ? 1 : q == 2 ? 0 : q == 3 ? 1 : 0) : (q == 0 ? 1 : 0);
}
__device__ __forceinline__ constexpr int prod_b(int x6, int q) {
    return x6 ? (q == 0 ? 0 : q == 1 ? 1 : q == 2 ? 2 : q == 3 ? 0 : q == 4 ? 1 : 0) : (q == 1 ? 1 : 0);
}

// ----------------------------------------------------------------------------- PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ long long gtime() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: false (and the error flag set) if the phase did not complete within `limit` ns, or if another
// thread already gave up. The clock and the flag (a global load) are checked once every 64 tries (each try returns
// within a bounded, system-dependent suspend time).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err, int code, long long limit) {
    if (mbar_try(bar, parity)) return true;
    const long long t0 = gtime();
    for (unsigned i = 1;; i++) {
        if (mbar_try(bar, parity)) return true;
        if ((i & 63u) == 0u && (gtime() - t0 > limit || *(volatile int*)err != 0)) {
            atomicCAS(err, 0, code);
            return false;
        }
    }
}
// After a wait gave up: wait (at most TC_DRAIN_NS, whatever the error flag says) for work this thread already
// started to land -- TMA loads into this block's shared memory, MMAs into its tensor memory -- so that the block
// neither exits nor frees its tensor memory with them in flight.
__device__ __forceinline__ void mbar_drain(uint32_t bar, uint32_t parity) {
    const long long t0 = gtime();
    for (unsigned i = 0;; i++) {
        if (mbar_try(bar, parity)) return;
        if ((i & 63u) == 63u && gtime() - t0 > TC_DRAIN_NS) return;
    }
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(dst), "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, uint32_t src, int x, int y, int z) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, %3}], [%4];"
                 ::"l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(src)
                 : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, uint32_t src, int x, int y) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];"
                 ::"l"((uint64_t)map), "r"(x), "r"(y), "r"(src)
                 : "memory");
}
__device__ __forceinline__ void st_shared_v4(uint32_t addr, float4 v) {
    asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}

// Shared-memory matrix descriptor: K-major tile of 128-byte rows, 128-byte swizzle, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFF) >> 4);        // start address
    d |= (uint64_t)1 << 16;                         // leading byte offset (unused by swizzled K-major tiles)
    d |= (uint64_t)(1024 >> 4) << 32;               // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1 << 46;                         // descriptor version of tcgen05
    d |= (uint64_t)2 << 61;                         // 128-byte swizzle
    return d;
}

// Operand kinds: A and B of one MMA always have the same type.
enum { KIND_BF16 = 0, KIND_F16 = 1, KIND_TF32 = 2 };

// Instruction descriptor: D float32; A and B both bf16 (format 1) or both float16 (format 0) for kind::f16, both tf32
// (format 2) for kind::tf32; both K-major; M = 128, N.
template <int N, int KIND>
__device__ __forceinline__ constexpr uint32_t idesc() {
    constexpr uint32_t fmt = KIND == KIND_BF16 ? 1u : KIND == KIND_F16 ? 0u : 2u;
    return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(TC_BM >> 4) << 24);
}

// One MMA: D (+)= A B^T over a K step of 32 bytes of the operand rows (16 elements of 16 bits, or 8 of tf32).
template <int N, int KIND>
__device__ __forceinline__ void mma_n(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
    if constexpr (KIND == KIND_TF32)
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
            ::"r"(tmem), "l"(a), "l"(b), "r"(idesc<N, KIND>()), "r"(accumulate));
    else
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
            ::"r"(tmem), "l"(a), "l"(b), "r"(idesc<N, KIND>()), "r"(accumulate));
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// Two 32-column loads in flight before one wait (columns taddr .. + 31 into v, taddr + 32 .. + 63 into u).
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, float (&v)[32], float (&u)[32]) {
    uint32_t r[32], q[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(q[0]), "=r"(q[1]), "=r"(q[2]), "=r"(q[3]), "=r"(q[4]), "=r"(q[5]), "=r"(q[6]), "=r"(q[7]),
          "=r"(q[8]), "=r"(q[9]), "=r"(q[10]), "=r"(q[11]), "=r"(q[12]), "=r"(q[13]), "=r"(q[14]), "=r"(q[15]),
          "=r"(q[16]), "=r"(q[17]), "=r"(q[18]), "=r"(q[19]), "=r"(q[20]), "=r"(q[21]), "=r"(q[22]), "=r"(q[23]),
          "=r"(q[24]), "=r"(q[25]), "=r"(q[26]), "=r"(q[27]), "=r"(q[28]), "=r"(q[29]), "=r"(q[30]), "=r"(q[31])
        : "r"(taddr + 32u));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) {
        v[i] = __uint_as_float(r[i]);
        u[i] = __uint_as_float(q[i]);
    }
}

// 1 / t for the field weights (t > 0 normal): the hardware approximation refined by one Newton-Raphson step,
// r' = r + r (1 - t r), within an ulp of the rounded reciprocal (the weights need float32 accuracy, not rounding).
__device__ __forceinline__ float recip(float t) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(t));
    return fmaf(r, fmaf(-t, r, 1.f), r);
}

// f16x3: the two float16 terms of x (already scaled into the chunk's range)
__device__ __forceinline__ void split2h(float x, __half& a, __half& b) {
    a = __float2half_rn(x);
    b = __float2half_rn(__fsub_rn(x, __half2float(a)));
}

__device__ __forceinline__ void split3(float v, __nv_bfloat16& a, __nv_bfloat16& b, __nv_bfloat16& c) {
    a = __float2bfloat16_rn(v);
    const float r1 = __fsub_rn(v, __bfloat162float(a));
    b = __float2bfloat16_rn(r1);
    c = __float2bfloat16_rn(__fsub_rn(r1, __bfloat162float(b)));
}

// ----------------------------------------------------------------------------- the GEMM kernel
// Warp roles (192 threads): warp 0 = TMA producer (and tensor-memory owner), warp 1 = MMA issuer, warps 2..5 =
// accumulator readers / epilogue (warp w reads tensor-memory lanes 32 (w % 4) .. + 31, i.e. output rows).
// The tensor cores accumulate in float32 with truncation, so a long accumulation drifts (about 2e-6 of the max
// after four chained GEMMs of K = 256). Each k-block (64 of K) therefore goes into a fresh tensor-memory
// accumulator (two, alternating) and the readers add it into float32 registers with round-to-nearest; the error
// then stays at float32 level (~2e-7) at every grid size.
constexpr int TC_THREADS = 192;

template <int BN, int EPI, int MODE>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap a0, const __grid_constant__ CUtensorMap b0,
                   const __grid_constant__ CUtensorMap a1, const __grid_constant__ CUtensorMap b1,
                   const __grid_constant__ CUtensorMap o0a, const __grid_constant__ CUtensorMap o0b,
                   const __grid_constant__ CUtensorMap o1a, const __grid_constant__ CUtensorMap o1b, TcArgs args) {
    // The set-up (barriers, tensor memory, tensor-map prefetch) reads nothing the previous kernel writes: it runs
    // before griddepcontrol.wait, overlapping the previous kernel's tail.
    constexpr int X6 = MODE == 1 ? 1 : 0;                        // bf16x6 (MODE 0: bf16x3, 2: f16x3, 3: tf32x3)
    constexpr bool F16 = MODE == 2;
    constexpr bool TF32 = MODE == 3;
    constexpr int KIND = TF32 ? KIND_TF32 : F16 ? KIND_F16 : KIND_BF16;
    constexpr int BKE = TF32 ? 32 : TC_BK;                       // elements of K per k-block (a 128-byte row)
    constexpr int B_TILE = BN * TC_BK * 2;
    constexpr int NA = X6 ? 3 : 2, NB = NA, NPROD = X6 ? 6 : 3;
    // bf16 modes, BN = 64: the products are grouped by B term into NBLK column blocks of the accumulator (block j =
    // the products with b_j), so that one MMA can cover several B terms at once (below). f16x3 and BN = 128: one
    // block, every product into it (the same tensor time: an MMA's time goes with its N; the readers load one block
    // per k-block instead of NB)
    constexpr bool CONCAT = BN == 64 && !F16;
    constexpr int NBLK = CONCAT ? NB : 1;
    constexpr uint32_t ACC_COLS = (uint32_t)(NBLK * BN);         // per accumulator buffer (two buffers)
    constexpr uint32_t TMEM_COLS = 2 * ACC_COLS <= 128 ? 128 : 2 * ACC_COLS <= 256 ? 256 : 512;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    // barriers: full[S], empty[S], acc_full[2], acc_empty[2]
    uint64_t* bars = (uint64_t*)(smem + TC_STAGE_SPACE);
    uint32_t* tmem_slot = (uint32_t*)(bars + 2 * TC_MAX_STAGES + 4);
    // f16x3: the factors of B's chunks, [K / 64][BN], each the upper half of the float32 2^(-F16_CONST - e) that takes
    // an accumulated product of a constant (times 2^F16_CONST) and a chunk scaled by 2^e back to its value (exact);
    // the table sits behind the stages (4 x 48 KB or 3 x 64 KB leave 24 KB of the stage space; checked on the host)
    constexpr int STAGE_BYTES = NA * TC_A_TILE + NB * B_TILE;
    constexpr int STAGES = TC_STAGE_SPACE / STAGE_BYTES > TC_MAX_STAGES ? TC_MAX_STAGES : TC_STAGE_SPACE / STAGE_BYTES;
    uint16_t* ftab = (uint16_t*)(smem + STAGES * STAGE_BYTES);   // (the host launches with args.stages = STAGES)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int z = blockIdx.z;
    const TcProblem& P = args.p[z];
    const CUtensorMap* ma = z ? &a1 : &a0;
    const CUtensorMap* mb = z ? &b1 : &b0;
    const int m0 = blockIdx.y * TC_BM, n0 = blockIdx.x * BN;
    const int total = P.K / BKE, stages = args.stages;
    constexpr int stage_bytes = NA * TC_A_TILE + NB * B_TILE;
    int* err = args.err;
    const long long limit = args.wait_ns;
    auto full_bar = [&](int s) { return smem_u32(&bars[s]); };
    auto empty_bar = [&](int s) { return smem_u32(&bars[TC_MAX_STAGES + s]); };
    auto accf_bar = [&](int b) { return smem_u32(&bars[2 * TC_MAX_STAGES + b]); };
    auto acce_bar = [&](int b) { return smem_u32(&bars[2 * TC_MAX_STAGES + 2 + b]); };

    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; s++) {
            mbar_init(full_bar(s), 1);
            mbar_init(empty_bar(s), 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(accf_bar(b), 1);
            mbar_init(acce_bar(b), 4);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();                                                // warp 0 converged for the .sync.aligned alloc
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 32) {
        for (const CUtensorMap* m : {ma, mb, z ? &o1a : &o0a, z ? &o1b : &o0b})
            asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)m) : "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    // The A operand of every GEMM of the field is one of its constant matrices, written by the field's set-up and
    // followed there by kernels that each wait for their predecessor: no kernel still running when this one starts
    // writes it. So the A tiles of the first stages are requested before the wait for the previous kernel (whose
    // outputs B is), and their latency overlaps that kernel's tail.
    const int pre = (args.early & 1) && !args.stall ? (total < stages ? total : stages) : 0;
    if (warp == 0 && lane == 0) {
        for (int it = 0; it < pre; it++) {                       // stage it, first use: no wait for a free stage
            mbar_expect_tx(full_bar(it), stage_bytes);
#pragma unroll
            for (int t = 0; t < NA; t++)
                tma_load_3d(smem_u32(smem + it * stage_bytes + t * TC_A_TILE), ma, full_bar(it), it * BKE, m0, t);
        }
    }
    pdl_wait();

    if (warp == 0) {
        if (lane == 0) {                                         // TMA producer
            int issued = 0;
            for (int it = 0; it < total && !args.stall; it++) {
                const int s = it % stages;
                const uint32_t ph = (uint32_t)(it / stages) & 1u;
                uint8_t* st = smem + s * stage_bytes;
                if (it >= pre) {                                 // (the first `pre` stages have their A already)
                    if (!mbar_wait(empty_bar(s), ph ^ 1u, err, 1, limit)) break;
                    mbar_expect_tx(full_bar(s), stage_bytes);
#pragma unroll
                    for (int t = 0; t < NA; t++)
                        tma_load_3d(smem_u32(st + t * TC_A_TILE), ma, full_bar(s), it * BKE, m0, t);
                }
#pragma unroll
                for (int t = 0; t < NB; t++) {
                    const uint32_t dst = smem_u32(st + NA * TC_A_TILE + t * B_TILE);
                    if (EPI == EPI_FOLD) {                       // B rows [64j, 64j + 64) and their mirror
                        tma_load_3d(dst, mb, full_bar(s), it * TC_BK, 64 * (int)blockIdx.x, t);
                        tma_load_3d(dst + 64 * 128, mb, full_bar(s), it * TC_BK, P.N - 64 - 64 * (int)blockIdx.x, t);
                    } else {
                        tma_load_3d(dst, mb, full_bar(s), it * BKE, n0, t);
                    }
                }
                issued = it + 1;
            }
            // a wait gave up (here or anywhere in the grid): the last load of each stage may still be in flight
            if (*(volatile int*)err != 0)
                for (int it = issued > stages ? issued - stages : 0; it < issued; it++)
                    mbar_drain(full_bar(it % stages), (uint32_t)(it / stages) & 1u);
        }
    } else if (warp == 1) {
        if (lane == 0) {                                         // MMA issuer: one k-block per accumulator
            int committed = 0;
            for (int it = 0; it < total; it++) {
                const int s = it % stages, b = it & 1;
                const uint32_t ph = (uint32_t)(it / stages) & 1u, use = (uint32_t)(it >> 1) & 1u;
                if (!mbar_wait(acce_bar(b), use ^ 1u, err, 2, limit)) break;
                if (!mbar_wait(full_bar(s), ph, err, 3, limit)) break;
                tc_fence_after();
                // descriptors of the stage's first A and B tiles; a tile or a 16-wide K step further on is the
                // same descriptor with its start-address field (address / 16) advanced (no carry: smem < 256 KB)
                const uint32_t st = smem_u32(smem + s * stage_bytes);
                const uint64_t da = smem_desc(st), db = smem_desc(st + NA * TC_A_TILE);
                const uint32_t acc = tmem + (uint32_t)b * ACC_COLS;
                auto A = [&](int t, int kk) { return da + (uint64_t)((t * TC_A_TILE + kk * 32) >> 4); };
                auto Bd = [&](int t, int kk) { return db + (uint64_t)((t * B_TILE + kk * 32) >> 4); };
                if constexpr (CONCAT) {
                    // B terms are consecutive tiles, so [b0 | b1 | b2] is one operand of N = 192 rows: a_i times
                    // several B terms is one MMA into consecutive blocks. Per block the order is still smallest
                    // product first, and each block starts fresh (accumulate = 0) with its first product.
                    if constexpr (X6) {
#pragma unroll
                        for (int kk = 0; kk < 4; kk++) mma_n<64, KIND>(acc, A(2, kk), Bd(0, kk), kk > 0);     // a2 b0
                        mma_n<64, KIND>(acc + 64, A(1, 0), Bd(1, 0), 0);                                      // a1 b1
                        mma_n<64, KIND>(acc, A(1, 0), Bd(0, 0), 1);                                           // a1 b0
#pragma unroll
                        for (int kk = 1; kk < 4; kk++) mma_n<128, KIND>(acc, A(1, kk), Bd(0, kk), 1);         // a1 [b0 b1]
                        mma_n<64, KIND>(acc + 128, A(0, 0), Bd(2, 0), 0);                                     // a0 b2
                        mma_n<128, KIND>(acc, A(0, 0), Bd(0, 0), 1);                                          // a0 [b0 b1]
#pragma unroll
                        for (int kk = 1; kk < 4; kk++) mma_n<192, KIND>(acc, A(0, kk), Bd(0, kk), 1);         // a0 [b0 b1 b2]
                    } else {
#pragma unroll
                        for (int kk = 0; kk < 4; kk++) mma_n<64, KIND>(acc, A(1, kk), Bd(0, kk), kk > 0);     // a1 b0
                        mma_n<64, KIND>(acc + 64, A(0, 0), Bd(1, 0), 0);                                      // a0 b1
                        mma_n<64, KIND>(acc, A(0, 0), Bd(0, 0), 1);                                           // a0 b0
#pragma unroll
                        for (int kk = 1; kk < 4; kk++) mma_n<128, KIND>(acc, A(0, kk), Bd(0, kk), 1);         // a0 [b0 b1]
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < NPROD; q++)
#pragma unroll
                        for (int kk = 0; kk < TC_BK / 16; kk++)
                            mma_n<BN, KIND>(acc, A(prod_a(X6, q), kk), Bd(prod_b(X6, q), kk), (q > 0 || kk > 0) ? 1u : 0u);
                }
                mma_commit(empty_bar(s));
                mma_commit(accf_bar(b));
                committed = it + 1;
            }
            // a wait gave up: the last commit tracks every MMA this thread issued; wait for it before the tensor
            // memory is freed
            if (*(volatile int*)err != 0 && committed > 0)
                mbar_drain(accf_bar((committed - 1) & 1), (uint32_t)((committed - 1) >> 1) & 1u);
        }
    } else {                                                     // readers + epilogue
        const int q4 = warp & 3;                                 // tensor-memory lane quarter
        const int row = m0 + q4 * 32 + lane;
        const float4 wr = EPI == EPI_WEIGHT2 ? P.wrow[P.m_out + row] : make_float4(0.f, 0.f, 0.f, 0.f);   // early
        if constexpr (F16) {                                     // this tile's factors of B, every k-block
            constexpr int wpk = BN / 4;                          // 4 exponents per global word
            const int rt = (int)threadIdx.x - 64, words = total * wpk;
            for (int w = rt; w < words; w += 128) {
                const int kb = w / wpk, c4 = w - kb * wpk;
                // (FOLD: columns 64 .. 127 are B rows N - 64j - 64 .. N - 64j - 1)
                const int n = EPI != EPI_FOLD ? n0 + 4 * c4
                              : 4 * c4 < 64 ? 64 * (int)blockIdx.x + 4 * c4 : P.N - 128 - 64 * (int)blockIdx.x + 4 * c4;
                const int e4 = __ldg((const int*)(P.b_exp + (size_t)kb * P.N + n));
                uint32_t f[4];
#pragma unroll
                for (int i = 0; i < 4; i++) f[i] = (uint32_t)(127 - F16_CONST - ((e4 << (24 - 8 * i)) >> 24)) << 7;
                ((uint2*)ftab)[w] = make_uint2(f[0] | (f[1] << 16), f[2] | (f[3] << 16));
            }
            asm volatile("bar.sync 1, 128;" ::: "memory");
        }
        constexpr bool MIRROR = EPI == EPI_MSPLIT || EPI == EPI_MPLAIN;
        float r[BN];
        float e[MIRROR ? BN : 1];                                // MIRROR: E, the sum over the first half of K
#pragma unroll
        for (int i = 0; i < BN; i++) r[i] = 0.f;
#pragma unroll
        for (int i = 0; i < (MIRROR ? BN : 1); i++) e[i] = 0.f;
        bool ok = true;
        for (int it = 0; it < total && ok; it++) {
            const int b = it & 1;
            if (MIRROR && it == total / 2) {                     // the even frequencies are summed: E aside, O next
#pragma unroll
                for (int i = 0; i < BN; i++) {
                    e[i] = r[i];
                    r[i] = 0.f;
                }
            }
            if (!mbar_wait(accf_bar(b), (uint32_t)(it >> 1) & 1u, err, 4, limit)) { ok = false; break; }
            tc_fence_after();
            const uint32_t base = tmem + ((uint32_t)(q4 * 32) << 16) + (uint32_t)b * ACC_COLS;
            // f16x3, 64 columns: both halves of the block in flight before one wait
            constexpr bool PAIR = F16 && BN == 64 && NBLK == 1;
            float v2[PAIR ? 32 : 1];
#pragma unroll
            for (int c0 = 0; c0 < BN; c0 += 32) {
                float v[32];
                if constexpr (PAIR) {
                    if (c0 == 0) tmem_ld64(base, v, v2);
                    else {
#pragma unroll
                        for (int i = 0; i < 32; i++) v[i] = v2[i];
                    }
                } else {
                    tmem_ld32(base + (uint32_t)c0, v);
                }
                if constexpr (NBLK > 1) {                        // blocks of the smaller products: add them first
                    float w[32];
                    tmem_ld32(base + (uint32_t)((NBLK - 1) * BN + c0), w);
                    if constexpr (NBLK > 2) {
                        float u[32];
                        tmem_ld32(base + (uint32_t)(BN + c0), u);
#pragma unroll
                        for (int i = 0; i < 32; i++) w[i] = __fadd_rn(w[i], u[i]);
                    }
#pragma unroll
                    for (int i = 0; i < 32; i++) v[i] = __fadd_rn(w[i], v[i]);
                }
                if constexpr (F16) {                             // back to values: exact powers of two
                    const uint32_t* tp = (const uint32_t*)(ftab + it * BN + c0);
#pragma unroll
                    for (int h = 0; h < 16; h++) {               // two factors per 4-byte read
                        const uint32_t w2 = tp[h];
                        r[c0 + 2 * h] = fmaf(v[2 * h], __uint_as_float(__byte_perm(w2, 0u, 0x1044u)), r[c0 + 2 * h]);
                        r[c0 + 2 * h + 1] =
                            fmaf(v[2 * h + 1], __uint_as_float(__byte_perm(w2, 0u, 0x3244u)), r[c0 + 2 * h + 1]);
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 32; i++) r[c0 + i] = __fadd_rn(r[c0 + i], v[i]);
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(acce_bar(b));
        }
        // the accumulation is done: a following GEMM may launch now (on the SMs this grid leaves free, and on each SM
        // as its block exits), so that its set-up and its constant loads overlap this epilogue
        if (args.early & 2) pdl_trigger();
        // Epilogue: the outputs go through shared memory (the stage buffers, idle now: every TMA load has been
        // consumed by a completed MMA) in the 128-byte-swizzled layout of 128-row x 128-byte boxes, and leave by
        // TMA stores, whole lines at a time (a thread holds one output row: direct stores would scatter 16-byte
        // pieces over 32 rows per instruction).
        ok = ok && *(volatile int*)err == 0;
        const int r_in = q4 * 32 + lane;                         // row inside the tile
        auto chunk = [&](int box, int c) {                       // byte offset of 16-byte chunk c of this row
            return (uint32_t)(box * EPI_BOX + r_in * 128 + ((c ^ (r_in & 7)) << 4));
        };
        const uint32_t sbase = smem_u32(smem);
        // the weighted epilogue's column weights: this tile's BN entries into shared memory (one wave of loads, read
        // back as broadcasts), behind the six output boxes
        constexpr int WSH_BOX = TF32 ? 8 : 6;                    // (tf32: Kx and Ky as 2 terms x 2 boxes each)
        const float4* wsh = (const float4*)(smem + WSH_BOX * EPI_BOX);
        if (EPI == EPI_WEIGHT2) {
            if (r_in < BN) ((float4*)(smem + WSH_BOX * EPI_BOX))[r_in] = P.wcol[n0 + r_in];
            asm volatile("bar.sync 1, 128;" ::: "memory");
        }
        // MIRROR: box row of this thread's row of the mirror tile (stored upside down: tile row r_in is output row
        // M_out - 1 - (om0 + r_in), box row 127 - r_in of a tile stored at M_out - om0 - 128)
        auto chunk_at = [&](int box, int c, bool mirror) {
            const int rr = mirror ? 127 - r_in : r_in;
            return (uint32_t)(box * EPI_BOX + rr * 128 + ((c ^ (rr & 7)) << 4));
        };
        if (ok) {
            if constexpr (MIRROR) {
                // row m = E + O (into e), its mirror msign (E - O) (into r); boxes from 0: the rows, behind them:
                // the mirror rows (float32: BN / 32 boxes each; float16: the 2 terms of the one 64-column chunk)
                const float sg = (float)P.msign;
#pragma unroll
                for (int i = 0; i < BN; i++) {
                    const float a = e[i], b = r[i];
                    e[i] = __fadd_rn(a, b);
                    r[i] = sg * __fsub_rn(a, b);
                }
                if (EPI == EPI_MPLAIN) {
#pragma unroll
                    for (int c = 0; c < BN / 4; c++) {
                        st_shared_v4(sbase + chunk_at(c >> 3, c & 7, false),
                                     make_float4(e[4 * c], e[4 * c + 1], e[4 * c + 2], e[4 * c + 3]));
                        st_shared_v4(sbase + chunk_at(BN / 32 + (c >> 3), c & 7, true),
                                     make_float4(r[4 * c], r[4 * c + 1], r[4 * c + 2], r[4 * c + 3]));
                    }
                } else {
                    auto put = [&](float (&v)[BN], int box0, bool mirror) {
                        float mx = 0.f;
#pragma unroll
                        for (int i = 0; i < BN; i++) mx = fmaxf(mx, fabsf(v[i]));
                        const int ex = f16_chunk_exp(mx);
                        const float sc = __int_as_float((127 + ex) << 23);
                        const int orow = mirror ? P.M_out - 1 - (P.m_out + row) : P.m_out + row;
                        P.o_exp[(size_t)(n0 / 64) * P.M_out + orow] = (signed char)ex;
#pragma unroll
                        for (int c = 0; c < 8; c++) {
                            __align__(16) __half ta[8], tb[8];
#pragma unroll
                            for (int i = 0; i < 8; i++) split2h(v[8 * c + i] * sc, ta[i], tb[i]);
                            st_shared_v4(sbase + chunk_at(box0, c, mirror), *(const float4*)ta);
                            st_shared_v4(sbase + chunk_at(box0 + 1, c, mirror), *(const float4*)tb);
                        }
                    };
                    put(e, 0, false);
                    put(r, 2, true);
                }
            } else if (EPI == EPI_PLAIN) {                       // float32: boxes of 32 columns
#pragma unroll
                for (int c = 0; c < BN / 4; c++)
                    st_shared_v4(sbase + chunk(c >> 3, c & 7), make_float4(r[4 * c], r[4 * c + 1], r[4 * c + 2],
                                                                          r[4 * c + 3]));
            } else if (EPI == EPI_FOLD) {
                // column c < 64 is B row 64j + c, column 127 - c its mirror N - 1 - (64j + c): sums into r[c],
                // differences into r[127 - c]; boxes 0-1: the terms of the sums, 2-3: of the differences, each the
                // output's 64-column chunk j with its own scale
#pragma unroll
                for (int c = 0; c < 64; c++) {
                    const float a = r[c], b = r[127 - c];
                    r[c] = __fadd_rn(a, b);
                    r[127 - c] = __fsub_rn(a, b);
                }
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    float mx = 0.f;
#pragma unroll
                    for (int i = 0; i < 64; i++) mx = fmaxf(mx, fabsf(r[64 * h + i]));
                    const int e = f16_chunk_exp(mx);
                    const float sc = __int_as_float((127 + e) << 23);
                    (h ? P.o2_exp : P.o_exp)[(size_t)blockIdx.x * P.M_out + P.m_out + row] = (signed char)e;
#pragma unroll
                    for (int c = 0; c < 8; c++) {
                        __align__(16) __half ta[8], tb[8];
#pragma unroll
                        for (int i = 0; i < 8; i++) split2h(r[h ? 127 - (8 * c + i) : 8 * c + i] * sc, ta[i], tb[i]);
                        st_shared_v4(sbase + chunk(2 * h, c), *(const float4*)ta);
                        st_shared_v4(sbase + chunk(2 * h + 1, c), *(const float4*)tb);
                    }
                }
            } else if (EPI == EPI_SPLIT && F16) {                // float16 terms of each 64-column chunk, scaled
#pragma unroll
                for (int g = 0; g < BN / 64; g++) {
                    float mx = 0.f;
#pragma unroll
                    for (int i = 0; i < 64; i++) mx = fmaxf(mx, fabsf(r[64 * g + i]));
                    const int e = f16_chunk_exp(mx);
                    const float sc = __int_as_float((127 + e) << 23);
                    P.o_exp[(size_t)(n0 / 64 + g) * P.M_out + P.m_out + row] = (signed char)e;
#pragma unroll
                    for (int c = 0; c < 8; c++) {
                        __align__(16) __half ta[8], tb[8];
#pragma unroll
                        for (int i = 0; i < 8; i++) split2h(r[64 * g + 8 * c + i] * sc, ta[i], tb[i]);
                        st_shared_v4(sbase + chunk(0 * (BN / 64) + g, c), *(const float4*)ta);
                        st_shared_v4(sbase + chunk(1 * (BN / 64) + g, c), *(const float4*)tb);
                    }
                }
            } else if (EPI == EPI_SPLIT && TF32) {               // tf32 terms (float32): boxes of 32 columns, term-major
#pragma unroll
                for (int c = 0; c < BN / 4; c++) {
                    float a[4], b[4];
#pragma unroll
                    for (int i = 0; i < 4; i++) {
                        a[i] = tf32_round(r[4 * c + i]);
                        b[i] = tf32_round(__fsub_rn(r[4 * c + i], a[i]));
                    }
                    const int g = c >> 3;
                    st_shared_v4(sbase + chunk(0 * (BN / 32) + g, c & 7), make_float4(a[0], a[1], a[2], a[3]));
                    st_shared_v4(sbase + chunk(1 * (BN / 32) + g, c & 7), make_float4(b[0], b[1], b[2], b[3]));
                }
            } else if (EPI == EPI_SPLIT) {                       // bf16 terms: boxes of 64 columns, term-major
#pragma unroll
                for (int c = 0; c < BN / 8; c++) {
                    __align__(16) __nv_bfloat16 ta[8], tb[8], tc[8];
#pragma unroll
                    for (int i = 0; i < 8; i++) split3(r[8 * c + i], ta[i], tb[i], tc[i]);
                    const int g = c >> 3;
                    st_shared_v4(sbase + chunk(0 * (BN / 64) + g, c & 7), *(const float4*)ta);
                    st_shared_v4(sbase + chunk(1 * (BN / 64) + g, c & 7), *(const float4*)tb);
                    st_shared_v4(sbase + chunk(2 * (BN / 64) + g, c & 7), *(const float4*)tc);
                }
            } else if (TF32) {
                // Kx = K Wx, Ky = K Wy (as below) in tf32 terms, boxes of 32 columns (BN = 64): 0-1 the first term of
                // Kx, 2-3 its second term, 4-7 the same for Ky
#pragma unroll
                for (int c = 0; c < BN / 4; c++) {
                    float xa[4], xb[4], ya[4], yb[4];
#pragma unroll
                    for (int i = 0; i < 4; i++) {
                        const float4 wc = wsh[4 * c + i];
                        const float t = wr.x + wc.x;
                        const float rr = t > 0.f ? recip(t) : 0.f;
                        const float kx = r[4 * c + i] * (wr.y * wc.z * rr), ky = r[4 * c + i] * (wc.y * wr.z * rr);
                        xa[i] = tf32_round(kx);
                        xb[i] = tf32_round(__fsub_rn(kx, xa[i]));
                        ya[i] = tf32_round(ky);
                        yb[i] = tf32_round(__fsub_rn(ky, ya[i]));
                    }
                    const int g = c >> 3;
                    st_shared_v4(sbase + chunk(0 * (BN / 32) + g, c & 7), make_float4(xa[0], xa[1], xa[2], xa[3]));
                    st_shared_v4(sbase + chunk(1 * (BN / 32) + g, c & 7), make_float4(xb[0], xb[1], xb[2], xb[3]));
                    st_shared_v4(sbase + chunk(2 * (BN / 32) + g, c & 7), make_float4(ya[0], ya[1], ya[2], ya[3]));
                    st_shared_v4(sbase + chunk(3 * (BN / 32) + g, c & 7), make_float4(yb[0], yb[1], yb[2], yb[3]));
                }
            } else if (F16) {
                // Kx = K Wx, Ky = K Wy as below, each row's 64 columns scaled by a power of two taken from an upper
                // bound of the row's magnitudes (a scale only has to keep the largest value under 2^15; a bound a
                // few thousand times too large still leaves it above 2^2, where float16 loses nothing that matters),
                // so that every product is formed once: |Kx| <= max|K| (s kx_p / bin_x) max w_q / t_min, |Ky| <=
                // max|K| w_p max(s ky_q / bin_x) / t_min, t_min the smallest kx_p^2 + ky_q^2 > 0 of the row in this
                // tile (the term with t = 0 is 0). Boxes 0-1: the terms of Kx, 2-3: of Ky.
                float cmin = INFINITY, cminpos = INFINITY, zmax = 0.f, ymax = 0.f;
#pragma unroll 8
                for (int i = 0; i < BN; i++) {
                    const float4 wc = wsh[i];
                    cmin = fminf(cmin, wc.x);
                    if (wc.x > 0.f) cminpos = fminf(cminpos, wc.x);
                    zmax = fmaxf(zmax, wc.z);
                    ymax = fmaxf(ymax, wc.y);
                }
                float mr = 0.f;
#pragma unroll
                for (int i = 0; i < BN; i++) mr = fmaxf(mr, fabsf(r[i]));
                const float tmin = wr.x > 0.f ? wr.x + cmin : cminpos;
                const float rt = tmin > 0.f && tmin < INFINITY ? recip(tmin) : 0.f;
                const int exx = f16_chunk_exp(mr * (wr.y * zmax) * rt), exy = f16_chunk_exp(mr * (ymax * wr.z) * rt);
                const float scx = __int_as_float((127 + exx) << 23), scy = __int_as_float((127 + exy) << 23);
                P.o_exp[(size_t)(n0 / 64) * P.M_out + P.m_out + row] = (signed char)exx;
                P.o2_exp[(size_t)(n0 / 64) * P.M_out + P.m_out + row] = (signed char)exy;
#pragma unroll
                for (int c = 0; c < BN / 8; c++) {
                    __align__(16) __half xa[8], xb[8], ya[8], yb[8];
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        const float4 wc = wsh[8 * c + i];
                        const float t = wr.x + wc.x;
                        const float rr = t > 0.f ? recip(t) : 0.f;
                        split2h(r[8 * c + i] * (wr.y * wc.z * rr) * scx, xa[i], xb[i]);
                        split2h(r[8 * c + i] * (wc.y * wr.z * rr) * scy, ya[i], yb[i]);
                    }
                    st_shared_v4(sbase + chunk(0, c), *(const float4*)xa);
                    st_shared_v4(sbase + chunk(1, c), *(const float4*)xb);
                    st_shared_v4(sbase + chunk(2, c), *(const float4*)ya);
                    st_shared_v4(sbase + chunk(3, c), *(const float4*)yb);
                }
            } else {
                // Kx = K Wx, Ky = K Wy with Wx = (s kx_p / bin_x) w_q r, Wy = (s ky_q / bin_x) w_p r,
                // r = 1 / (kx_p^2 + ky_q^2) (0 at p = q = 0), from per-row and per-column tables; boxes 0-2: the
                // terms of Kx, 3-5: of Ky (BN = 64: one box per term)
#pragma unroll
                for (int c = 0; c < BN / 8; c++) {
                    __align__(16) __nv_bfloat16 xa[8], xb[8], xc[8], ya[8], yb[8], yc[8];
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        const float4 wc = wsh[8 * c + i];
                        const float t = wr.x + wc.x;
                        const float rr = t > 0.f ? recip(t) : 0.f;
                        split3(r[8 * c + i] * (wr.y * wc.z * rr), xa[i], xb[i], xc[i]);
                        split3(r[8 * c + i] * (wc.y * wr.z * rr), ya[i], yb[i], yc[i]);
                    }
                    st_shared_v4(sbase + chunk(0, c), *(const float4*)xa);
                    st_shared_v4(sbase + chunk(1, c), *(const float4*)xb);
                    st_shared_v4(sbase + chunk(2, c), *(const float4*)xc);
                    st_shared_v4(sbase + chunk(3, c), *(const float4*)ya);
                    st_shared_v4(sbase + chunk(4, c), *(const float4*)yb);
                    st_shared_v4(sbase + chunk(5, c), *(const float4*)yc);
                }
            }
        }
        // every reader thread reaches this barrier (all its waits above are bounded), whatever `ok` says
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("bar.sync 1, 128;" ::: "memory");
        if (warp == 2 && lane == 0 && *(volatile int*)err == 0) {
            const int om0 = m0 + P.m_out;         // the tile's first output row
            const CUtensorMap* mo = z ? &o1a : &o0a;
            const CUtensorMap* mo2 = z ? &o1b : &o0b;
            if (EPI == EPI_MPLAIN || EPI == EPI_MSPLIT) {
                const int mm0 = P.M_out - om0 - TC_BM;          // the mirror tile (rows upside down in its boxes)
                if (EPI == EPI_MPLAIN) {
#pragma unroll
                    for (int b = 0; b < BN / 32; b++) {
                        tma_store_2d(mo, sbase + b * EPI_BOX, n0 + 32 * b, om0);
                        tma_store_2d(mo, sbase + (BN / 32 + b) * EPI_BOX, n0 + 32 * b, mm0);
                    }
                } else {
#pragma unroll
                    for (int t = 0; t < 2; t++) {
                        tma_store_3d(mo, sbase + t * EPI_BOX, n0, om0, t);
                        tma_store_3d(mo, sbase + (2 + t) * EPI_BOX, n0, mm0, t);
                    }
                }
            } else if (EPI == EPI_PLAIN) {
#pragma unroll
                for (int b = 0; b < BN / 32; b++) tma_store_2d(mo, sbase + b * EPI_BOX, n0 + 32 * b, om0);
            } else if (EPI == EPI_FOLD) {
#pragma unroll
                for (int t = 0; t < 2; t++) {
                    tma_store_3d(mo, sbase + t * EPI_BOX, 64 * (int)blockIdx.x, om0, t);
                    tma_store_3d(mo2, sbase + (2 + t) * EPI_BOX, 64 * (int)blockIdx.x, om0, t);
                }
            } else if (EPI == EPI_SPLIT && TF32) {               // 2 terms of BN / 32 boxes of 32 float32 columns
#pragma unroll
                for (int t = 0; t < 2; t++)
#pragma unroll
                    for (int g = 0; g < BN / 32; g++)
                        tma_store_3d(mo, sbase + (t * (BN / 32) + g) * EPI_BOX, n0 + 32 * g, om0, t);
            } else if (EPI == EPI_SPLIT) {
                constexpr int OT = F16 ? 2 : 3;                  // output terms
#pragma unroll
                for (int t = 0; t < OT; t++)
#pragma unroll
                    for (int g = 0; g < BN / 64; g++) tma_store_3d(mo, sbase + (t * (BN / 64) + g) * EPI_BOX, n0 + 64 * g, om0, t);
            } else if (TF32) {                                   // WEIGHT2: Kx, Ky: 2 terms x BN / 32 boxes each
#pragma unroll
                for (int t = 0; t < 2; t++)
#pragma unroll
                    for (int g = 0; g < BN / 32; g++) {
                        tma_store_3d(mo, sbase + (t * (BN / 32) + g) * EPI_BOX, n0 + 32 * g, om0, t);
                        tma_store_3d(mo2, sbase + ((2 + t) * (BN / 32) + g) * EPI_BOX, n0 + 32 * g, om0, t);
                    }
            } else {
                constexpr int OT = F16 ? 2 : 3;
#pragma unroll
                for (int t = 0; t < OT; t++) {
                    tma_store_3d(mo, sbase + t * EPI_BOX, n0, om0, t);
                    tma_store_3d(mo2, sbase + (OT + t) * EPI_BOX, n0, om0, t);
                }
            }
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            // wait until the stores have read the staged boxes (the shared memory may then go); their writes are
            // visible to the next kernel when this grid completes, which its griddepcontrol.wait waits for
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        }
    }
    // Lane 0 of warps 0 and 1 leaves its role loop long after the other 31 lanes: reconverge every warp before the
    // block barrier (an aligned barrier reached by a diverged warp can let the block through early), so that the
    // tensor memory is freed only after every MMA has completed and every reader is done.
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

// ----------------------------------------------------------------------------- host side
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

// Term planes [terms][rows][K] as a 3-D tensor (K, rows, term); box = one 128-byte row of K x box_rows x 1. Three
// bf16 planes (the bf16 modes; bf16x3 reads two of them), two float16 planes (f16x3, MODE 2) or two float32 planes
// holding tf32 terms (tf32x3, MODE 3: a box row is 32 elements).
static bool make_map(CUtensorMap* m, const void* base, int rows, int K, int box_rows, int mode = 0) {
    auto fn = encode_fn();
    if (!fn) return false;
    const bool f16 = mode == 2, tf = mode == 3;
    const cuuint64_t es = tf ? 4 : 2;
    cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, f16 || tf ? 2u : 3u};
    cuuint64_t strides[2] = {(cuuint64_t)K * es, (cuuint64_t)rows * K * es};
    cuuint32_t box[3] = {(cuuint32_t)(128 / es), (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(m, tf ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : f16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                                  : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3,
                    const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// A float32 plane [rows][cols] as a 2-D tensor; box = 32 columns (128 bytes) x 128 rows, 128-byte swizzle.
static bool make_map_f32(CUtensorMap* m, const void* base, int rows, int cols) {
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * 4};
    cuuint32_t box[2] = {32, (cuuint32_t)TC_BM};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

bool field_tc_supported(int nbx, int nby) {
    return nbx >= 128 && nby >= 128 && nbx % 128 == 0 && nby % 128 == 0 && nbx <= 4096 && nby <= 4096;
}

struct TcOp {
    const void* a; int arows;
    const void* b; int brows;
    TcProblem p;
};

template <int BN, int EPI, int MODE>
static int launch_tc_mode(const TcOp* ops, int nops, int* err, cudaStream_t s, int early) {
    constexpr bool F16 = MODE == 2;
    // the shared-memory attribute is a property of the function on each device: set once per device (a race of two
    // host threads sets it twice, which is harmless)
    static unsigned long long attr_set[4] = {0, 0, 0, 0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return GP103_ERR_CUDA;
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(__atomic_load_n(&attr_set[dev >> 6], __ATOMIC_ACQUIRE) & bit)) {
        if (cudaFuncSetAttribute(tc_gemm_kernel<BN, EPI, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM) !=
            cudaSuccess)
            return GP103_ERR_CUDA;
        __atomic_fetch_or(&attr_set[dev >> 6], bit, __ATOMIC_ACQ_REL);
    }
    constexpr int terms = MODE == 1 ? 3 : 2;
    constexpr int stage_bytes = terms * TC_A_TILE + terms * BN * TC_BK * 2;
    constexpr int stages = TC_STAGE_SPACE / stage_bytes > TC_MAX_STAGES ? TC_MAX_STAGES : TC_STAGE_SPACE / stage_bytes;
    CUtensorMap maps[8];
    TcArgs args = {};
    for (int z = 0; z < 2; z++) {
        const TcOp& o = ops[z < nops ? z : 0];
        if (F16 && ((long long)(o.p.K / TC_BK) * BN * 2 > TC_STAGE_SPACE - (long long)stages * stage_bytes ||
                    !o.p.b_exp || (EPI != EPI_PLAIN && EPI != EPI_MPLAIN && !o.p.o_exp) ||
                    ((EPI == EPI_WEIGHT2 || EPI == EPI_FOLD) && !o.p.o2_exp)))
            return GP103_ERR_ARG;
        if (!make_map(&maps[2 * z], o.a, o.arows, o.p.K, TC_BM, MODE) ||
            !make_map(&maps[2 * z + 1], o.b, o.brows, o.p.K, EPI == EPI_FOLD ? 64 : BN, MODE))
            return GP103_ERR_CUDA;
        // outputs (stored by TMA): bf16 terms [3][M][N] as (N, M, term) boxes of 64 x 128; float32 [M][N]
        CUtensorMap* oa = &maps[4 + 2 * z];
        CUtensorMap* ob = &maps[5 + 2 * z];
        bool ok = true;
        if (EPI == EPI_PLAIN || EPI == EPI_MPLAIN) {
            ok = make_map_f32(oa, o.p.out_f32, o.p.M_out, o.p.N);
            *ob = *oa;
        } else {
            const int ncols = EPI == EPI_FOLD ? o.p.N / 2 : o.p.N;
            ok = make_map(oa, o.p.o_terms, o.p.M_out, ncols, TC_BM, MODE);
            if (ok && (EPI == EPI_WEIGHT2 || EPI == EPI_FOLD)) ok = make_map(ob, o.p.o2_terms, o.p.M_out, ncols, TC_BM, MODE);
            else *ob = *oa;
        }
        if (!ok) return GP103_ERR_CUDA;
        args.p[z] = o.p;
    }
    args.stages = stages;
    args.err = err;
    args.wait_ns = tc_wait_ns();
    args.stall = tc_test_stall() ? 1 : 0;
    args.early = early;
    const TcProblem& p = ops[0].p;
    dim3 grid(p.N / BN, p.M / TC_BM, nops);
    if (launch_k(tc_gemm_kernel<BN, EPI, MODE>, dim3(grid), dim3(TC_THREADS), TC_SMEM, s, maps[0], maps[1], maps[2],
                 maps[3], maps[4], maps[5], maps[6], maps[7], args) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

template <int BN, int EPI>
static int launch_tc_bn(const TcOp* ops, int nops, int mode, int* err, cudaStream_t s, int early) {
    if (mode == GP103_FIELD_BF16X3) return launch_tc_mode<BN, EPI, 0>(ops, nops, err, s, early);
    if (mode == GP103_FIELD_F16X3) return launch_tc_mode<BN, EPI, 2>(ops, nops, err, s, early);
    if (mode == GP103_FIELD_TF32X3) return launch_tc_mode<BN, EPI, 3>(ops, nops, err, s, early);
    return launch_tc_mode<BN, EPI, 1>(ops, nops, err, s, early);
}

// One GEMM per launch: 64-column tiles (twice the blocks); two per launch: 128-column tiles, or 64-column ones
// (bn = 64: two half-height problems). The epilogue is a template argument (every problem of a launch has the same
// one). `last`: no GEMM of the field follows this launch (it then does not let the next kernel launch early).
static int launch_tc(const TcOp* ops, int nops, int mode, int* err, cudaStream_t s, int bn = 0, bool last = false) {
    const int epi = ops[0].p.epi;
    const int early = field_early() & (last ? 1 : 3);
    if (epi == EPI_SPLIT && (nops == 1 || bn == 64)) return launch_tc_bn<64, EPI_SPLIT>(ops, nops, mode, err, s, early);
    if (epi == EPI_WEIGHT2 && (nops == 1 || bn == 64))
        return launch_tc_bn<64, EPI_WEIGHT2>(ops, nops, mode, err, s, early);
    if (epi == EPI_FOLD)                                         // 128 columns: 64 and their mirror (f16x3 only)
        return mode == GP103_FIELD_F16X3 ? launch_tc_mode<128, EPI_FOLD, 2>(ops, nops, err, s, early) : GP103_ERR_ARG;
    if (epi == EPI_MSPLIT)                                       // half-height tiles, each with its mirror (f16x3)
        return mode == GP103_FIELD_F16X3 ? launch_tc_mode<64, EPI_MSPLIT, 2>(ops, nops, err, s, early) : GP103_ERR_ARG;
    if (epi == EPI_MPLAIN)
        return mode == GP103_FIELD_F16X3 ? launch_tc_mode<64, EPI_MPLAIN, 2>(ops, nops, err, s, early) : GP103_ERR_ARG;
    if (nops == 2 && epi == EPI_SPLIT) return launch_tc_bn<128, EPI_SPLIT>(ops, nops, mode, err, s, early);
    if (nops == 2 && epi == EPI_PLAIN) return launch_tc_bn<128, EPI_PLAIN>(ops, nops, mode, err, s, early);
    return GP103_ERR_ARG;                                        // no other combination is used
}

__global__ void split_density_kernel(const float* d, size_t n, float shift, __nv_bfloat16* t) {
    pdl_wait();
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        __nv_bfloat16 a, b, c;
        split3(__fsub_rn(d[e], shift), a, b, c);
        t[e] = a;
        t[n + e] = b;
        t[2 * n + e] = c;
    }
}

// tf32x3: the shifted float32 density into two tf32 terms (float32 planes t[0 .. n), t[n .. 2n))
__global__ void split_density_tf32_kernel(const float* d, size_t n, float shift, float* t) {
    pdl_wait();
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const float x = __fsub_rn(d[e], shift), a = tf32_round(x);
        t[e] = a;
        t[n + e] = tf32_round(__fsub_rn(x, a));
    }
}

// f16x3: a float32 density [nbx][nby] into two float16 terms, each row's 64-bin chunks scaled by their own power of
// two (one warp per chunk, two bins per lane), the exponents in e[(y / 64) * nbx + x]
__global__ void split_density_f16_kernel(const float* d, int nbx, int nby, float shift, __half* t, signed char* e) {
    pdl_wait();
    const int lane = threadIdx.x & 31;
    const long long chunks = (long long)nbx * nby / 64, n = (long long)nbx * nby;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long c = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); c < chunks; c += warps) {
        float2 v = *(const float2*)(d + 64 * c + 2 * lane);
        v.x = __fsub_rn(v.x, shift);
        v.y = __fsub_rn(v.y, shift);
        float mx = fmaxf(fabsf(v.x), fabsf(v.y));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        const int ex = f16_chunk_exp(mx);
        const float sc = __int_as_float((127 + ex) << 23);
        __half a0, b0, a1, b1;
        split2h(v.x * sc, a0, b0);
        split2h(v.y * sc, a1, b1);
        *(__half2*)(t + 64 * c + 2 * lane) = __halves2half2(a0, a1);
        *(__half2*)(t + n + 64 * c + 2 * lane) = __halves2half2(b0, b1);
        if (lane == 0) {
            const long long x = (64 * c) / nby, y = (64 * c) % nby;
            e[(y / 64) * nbx + x] = (signed char)ex;
        }
    }
}

// f16x3 folded: a float32 density [nbx][nby] folded about the middle of y, s = d(y) + d(nby-1-y) and
// t = d(y) - d(nby-1-y) for y < nby/2, each [nbx][nby/2] as two float16 terms per 64-value chunk of a row scaled by
// its own power of two (one warp per chunk of s and the same chunk of t, two values per lane): planes s0, s1, t0, t1
// of nbx * nby/2 values from `out` on; exponents of s in e[(y / 64) * nbx + x] (y < nby/2), of t behind them.
__global__ void split_density_fold_kernel(const float* d, int nbx, int nby, float shift, __half* out,
                                          signed char* e) {
    pdl_wait();
    const int lane = threadIdx.x & 31, hy = nby / 2;
    const long long chunks = (long long)nbx * hy / 64, hn = (long long)nbx * hy;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long c = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); c < chunks; c += warps) {
        const long long x = (64 * c) / hy;
        const int y = (int)((64 * c) % hy) + 2 * lane;
        const float* row = d + x * nby;
        const float2 lo = *(const float2*)(row + y);
        const float h0 = row[nby - 1 - y], h1 = row[nby - 2 - y];
        const float s0 = __fadd_rn(__fsub_rn(lo.x, shift), __fsub_rn(h0, shift));
        const float s1 = __fadd_rn(__fsub_rn(lo.y, shift), __fsub_rn(h1, shift));
        const float t0 = __fsub_rn(lo.x, h0), t1 = __fsub_rn(lo.y, h1);
        float ms = fmaxf(fabsf(s0), fabsf(s1)), mt = fmaxf(fabsf(t0), fabsf(t1));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            ms = fmaxf(ms, __shfl_xor_sync(0xffffffffu, ms, o));
            mt = fmaxf(mt, __shfl_xor_sync(0xffffffffu, mt, o));
        }
        const int es = f16_chunk_exp(ms), et = f16_chunk_exp(mt);
        const float scs = __int_as_float((127 + es) << 23), sct = __int_as_float((127 + et) << 23);
        __half a0, b0, a1, b1;
        const long long at = x * hy + y;
        split2h(s0 * scs, a0, b0);
        split2h(s1 * scs, a1, b1);
        *(__half2*)(out + at) = __halves2half2(a0, a1);
        *(__half2*)(out + hn + at) = __halves2half2(b0, b1);
        split2h(t0 * sct, a0, b0);
        split2h(t1 * sct, a1, b1);
        *(__half2*)(out + 2 * hn + at) = __halves2half2(a0, a1);
        *(__half2*)(out + 3 * hn + at) = __halves2half2(b0, b1);
        if (lane == 0) {
            const long long k = (long long)(y / 64) * nbx + x;
            e[k] = (signed char)es;
            e[(long long)(hy / 64) * nbx + k] = (signed char)et;
        }
    }
}

int field_tc(const FieldLayout& L, const void* cbuf, void* wbuf, const float* density, float* ex, float* ey,
             cudaStream_t s) {
    if (!field_tc_supported(L.nbx, L.nby)) return GP103_ERR_SHAPE;
    const char* c = (const char*)cbuf;
    char* w = (char*)wbuf;
    const int X = L.nbx, Y = L.nby;
    auto B = [](const char* base, size_t off) { return (__nv_bfloat16*)(base + off); };
    int* err = (int*)(w + L.w_err);
    int st;
    const bool f16 = L.mode == GP103_FIELD_F16X3;
    auto E = [&](size_t off) { return f16 ? (signed char*)(w + off) : (signed char*)nullptr; };
    if (density && L.fold) {
        if (launch_k(split_density_fold_kernel, dim3(grid_for((size_t)X * Y / 4, 256, 8)), dim3(256), 0, s, density,
                     X, Y, L.shift, (__half*)(w + L.w_a), E(L.e_a)) != cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    } else if (density && L.mode == GP103_FIELD_TF32X3) {
        if (launch_k(split_density_tf32_kernel, dim3(grid_for((size_t)X * Y, 256, 8)), dim3(256), 0, s, density,
                     (size_t)X * Y, L.shift, (float*)(w + L.w_a)) != cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    } else if (density && f16) {
        if (launch_k(split_density_f16_kernel, dim3(grid_for((size_t)X * Y / 2, 256, 8)), dim3(256), 0, s, density, X,
                     Y, L.shift, (__half*)(w + L.w_a), E(L.e_a)) != cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    } else if (density) {
        if (launch_k(split_density_kernel, dim3(grid_for((size_t)X * Y, 256, 8)), dim3(256), 0, s, density,
                     (size_t)X * Y, L.shift, B(w, L.w_a)) != cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    }
    auto prob = [](int M, int N, int K, int epi) {
        TcProblem p = {};
        p.M = M; p.N = N; p.K = K; p.epi = epi;
        p.M_out = M;
        return p;
    };
    // 1: Tt = (A Cy^T)^T = Cy A^T: Cy as the row operand, the density as the column operand, so the transposed
    //    product comes out in rows (no transposing epilogue); folded (f16x3): rows in the folded frequency order, which
    //    K's columns, the column weights and the A operands CyT / SyT of step 3 follow
    if (L.fold) {
        // folded (f16x3). 1: the even frequencies of the density's folded sum and the odd ones of its folded
        // difference (two GEMMs of half the height and half the depth in one launch), rows [0, Y/2) / [Y/2, Y) of Tt,
        // the epilogue folding Tt about the middle of x: sums Ts and differences Td, [2 terms][Y][X/2] each
        const int H = Y / 2, G = X / 2;
        const size_t cy_half = (size_t)H * H * 2, a_half = (size_t)X * H * 2, t_half = (size_t)Y * G * 2;
        TcOp o1[2] = {{B(c, L.c_cy), H, B(w, L.w_a), X, prob(H, X, H, EPI_FOLD)},
                      {B(c, L.c_cy) + cy_half, H, B(w, L.w_a) + a_half, X, prob(H, X, H, EPI_FOLD)}};
        for (int z = 0; z < 2; z++) {
            o1[z].p.o_terms = B(w, L.w_tt);
            o1[z].p.o2_terms = B(w, L.w_tt) + t_half;
            o1[z].p.M_out = Y;
            o1[z].p.m_out = z * H;
            o1[z].p.b_exp = E(L.e_a) + (size_t)z * (H / 64) * X;
            o1[z].p.o_exp = E(L.e_tt);
            o1[z].p.o2_exp = E(L.e_tt) + (size_t)(G / 64) * Y;
        }
        if ((st = launch_tc(o1, 2, L.mode, err, s))) return st;
        // 2: the even frequencies along x from Ts and the odd ones from Td, rows [0, X/2) / [X/2, X) of K, weighted
        const size_t cx_half = (size_t)G * G * 2;
        TcOp o2[2] = {{B(c, L.c_cx), G, B(w, L.w_tt), Y, prob(G, Y, G, EPI_WEIGHT2)},
                      {B(c, L.c_cx) + cx_half, G, B(w, L.w_tt) + t_half, Y, prob(G, Y, G, EPI_WEIGHT2)}};
        for (int z = 0; z < 2; z++) {
            o2[z].p.o_terms = B(w, L.w_kx);
            o2[z].p.o2_terms = B(w, L.w_ky);
            o2[z].p.M_out = X;
            o2[z].p.m_out = z * G;
            o2[z].p.b_exp = E(L.e_tt) + (size_t)z * (G / 64) * Y;
            o2[z].p.o_exp = E(L.e_kx);
            o2[z].p.o2_exp = E(L.e_ky);
            o2[z].p.wrow = (const float4*)(c + L.c_wrow);
            o2[z].p.wcol = (const float4*)(c + L.c_wcol);
        }
        if ((st = launch_tc(o2, 2, L.mode, err, s, 64))) return st;
    } else {
        TcOp o1 = {B(c, L.c_cy), Y, B(w, L.w_a), X, prob(Y, X, Y, EPI_SPLIT)};
        o1.p.o_terms = B(w, L.w_tt);
        o1.p.b_exp = E(L.e_a);
        o1.p.o_exp = E(L.e_tt);
        if ((st = launch_tc(&o1, 1, L.mode, err, s))) return st;
        // 2: K = Cx T -> Kx, Ky
        TcOp o2 = {B(c, L.c_cx), X, B(w, L.w_tt), Y, prob(X, Y, X, EPI_WEIGHT2)};
        o2.p.o_terms = B(w, L.w_kx);
        o2.p.o2_terms = B(w, L.w_ky);
        o2.p.b_exp = E(L.e_tt);
        o2.p.o_exp = E(L.e_kx);
        o2.p.o2_exp = E(L.e_ky);
        o2.p.wrow = (const float4*)(c + L.c_wrow);
        o2.p.wcol = (const float4*)(c + L.c_wcol);
        if ((st = launch_tc(&o2, 1, L.mode, err, s))) return st;
    }
    // 3a / 4a: Pt = (Kx Cy)^T = Cy^T Kx^T, Qt = (Ky Sy)^T = Sy^T Ky^T (row operand Cy^T / Sy^T, column operand Kx / Ky);
    // folded: rows n < Y/2 and their mirrors Y-1-n from the even and odd frequencies (cosine: E - O, sine: O - E)
    const int e3 = L.fold ? EPI_MSPLIT : EPI_SPLIT, M3 = L.fold ? Y / 2 : Y;
    TcOp o3[2] = {{B(c, L.c_cyt), Y, B(w, L.w_kx), X, prob(M3, X, Y, e3)},
                  {B(c, L.c_syt), Y, B(w, L.w_ky), X, prob(M3, X, Y, e3)}};
    o3[0].p.M_out = o3[1].p.M_out = Y;
    o3[0].p.msign = 1;
    o3[1].p.msign = -1;
    o3[0].p.o_terms = B(w, L.w_pt);
    o3[1].p.o_terms = B(w, L.w_qt);
    o3[0].p.b_exp = E(L.e_kx);
    o3[0].p.o_exp = E(L.e_pt);
    o3[1].p.b_exp = E(L.e_ky);
    o3[1].p.o_exp = E(L.e_qt);
    if ((st = launch_tc(o3, 2, L.mode, err, s))) return st;
    // 3b / 4b: Ex = Sx^T P, Ey = Cx^T Q (folded: as step 3, rows m < X/2 and their mirrors)
    const int e4 = L.fold ? EPI_MPLAIN : EPI_PLAIN, M4 = L.fold ? X / 2 : X;
    TcOp o4[2] = {{B(c, L.c_sxt), X, B(w, L.w_pt), Y, prob(M4, Y, X, e4)},
                  {B(c, L.c_cxt), X, B(w, L.w_qt), Y, prob(M4, Y, X, e4)}};
    o4[0].p.M_out = o4[1].p.M_out = X;
    o4[0].p.msign = -1;
    o4[1].p.msign = 1;
    o4[0].p.out_f32 = ex;
    o4[1].p.out_f32 = ey;
    o4[0].p.b_exp = E(L.e_pt);
    o4[1].p.b_exp = E(L.e_qt);
    return launch_tc(o4, 2, L.mode, err, s, 0, true);
}

}  // namespace gp103
