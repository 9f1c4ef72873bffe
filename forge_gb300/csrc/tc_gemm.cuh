// tcgen05 (5th-generation tensor core) GEMM for sm_103a, TF32 inputs, FP32 results.
//
//   D[b](m, n) = sum_k A[b](m, k) * B[b](n, k)        (both operands K-major, fp32 storage read as tf32)
//
// One CTA (192 threads) per 128 x 64 output tile:
//   warp 0 / lane 0 : TMA producer (cp.async.bulk.tensor.3d, 128B swizzle, 4-stage ring)
//   warp 1 / lane 0 : MMA issuer   (tcgen05.mma.cta_group::1.kind::tf32, M=128 N=64 K=8); warp 1
//                     also allocates and frees the TMEM
//   warps 2..5      : accumulators (tcgen05.ld.32x32b.x32 -> FP32 registers) and epilogue
// The tensor core's FP32 accumulation truncates (measured: an all-positive K = 8192 product comes
// out 5.9e-5 low, linearly in K), so each K block of 32 is accumulated alone into one of two TMEM
// buffers (64 columns each) and added into round-to-nearest FP32 registers by warps 2..5 while the
// MMAs of the next block run in the other buffer: the residual bias is that of 4 MMAs.
// Every mbarrier wait is bounded; on timeout the kernel raises an error flag, stops issuing,
// drains, frees its TMEM and returns.
//
// Complex products run as real GEMMs over operands staged by the callers (real/imag planes,
// and hi/lo TF32 splits for FP32-accurate results: a*b ~ ah*bh + ah*bl + al*bh).
//
// Exact-block mode (FLUSH > 1, DF = true; the sliced products of the eigenpair refinement):
// the operands are integer slices |s| <= 256 (Ozaki et al., "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and its applications",
// Numer. Algorithms 59, 2012), so a K block of FLUSH x 32 <= 256 products sums to an integer
// below 2^24 and TMEM holds it exactly.  Each such block is scaled by 2^-sexp[segment] (exact)
// and added into double-float (hi, lo) registers with an error-free TwoSum; the epilogue gets
// hi + lo as doubles.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "forge_internal.cuh"

namespace forge {

// 4 stages x 24 KB + barriers and 128 TMEM columns per CTA keep two CTAs resident per SM.
constexpr int TC_BM = 128, TC_BN = 64, TC_BK = 32, TC_STAGES = 4, TC_THREADS = 192;
constexpr int TC_A_BYTES = TC_BM * TC_BK * 4;  // 16 KB per stage
constexpr int TC_B_BYTES = TC_BN * TC_BK * 4;  //  8 KB per stage
constexpr int TC_SMEM = TC_STAGES * (TC_A_BYTES + TC_B_BYTES) + 1024 + 256;
constexpr uint32_t TC_TMEM_COLS = 2 * TC_BN;     // two accumulation buffers
constexpr uint32_t TC_SPIN_LIMIT = 1u << 26;     // bounded waits (>> any legitimate wait)

struct TcOperand {
    const float* ptr;
    int64_t rows, cols;      // rows = M (or N), cols = K extent of one plane (elements, contiguous)
    int64_t ld;              // row pitch in elements (multiple of 4)
    int64_t batch_stride;    // elements between planes (3rd TMA dimension)
    int64_t nplanes = 0;     // extent of the 3rd dimension (0: = batch)
};

// K-block -> TMA coordinate map of one operand.  The GEMM's K runs over nseg segments of
// nkp blocks of 32; segment s reads plane zsel[s] (+ zbatch * batch index) starting at
// element koff of each row.  A plain operand is nseg = 1, zsel = {0}, zbatch = 1.
constexpr int TC_MAXSEG = 32;
struct TcKMap {
    int32_t nkp, nseg, koff, zbatch;
    int32_t zsel[TC_MAXSEG];
    int8_t sexp[TC_MAXSEG];   // exact-block mode: segment s is scaled by 2^-sexp[s] (A map)
};

__host__ __device__ inline TcKMap tc_kmap_plain(int64_t K) {
    TcKMap m{};
    m.nkp = (int32_t)((K + 31) / 32);
    m.nseg = 1;
    m.koff = 0;
    m.zbatch = 1;
    return m;
}

// Builds the 3D TMA descriptor {K, rows, planes} with a 32 x box_rows box and 128B swizzle.
int tc_make_tmap(CUtensorMap* map, const TcOperand& op, int64_t batch, int box_rows);

__device__ inline uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ inline void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ inline void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ inline void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Failure-injection controls of one launch (test hooks): the iteration bound of every mbarrier
// wait, and a K block at which the TMA producer stops issuing (-1: never), so that the MMA issuer's
// wait for that block runs out.  Normal launches use {TC_SPIN_LIMIT, -1}.
struct TcFault {
    uint32_t spin_limit = TC_SPIN_LIMIT;
    int32_t stop_loads_at = -1;
};

// returns false if the wait gave up
__device__ inline bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                 uint32_t limit = TC_SPIN_LIMIT) {
    uint32_t done = 0;
    for (uint32_t it = 0; it < limit; ++it) {
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (abort_flag && (it & 1023u) == 1023u && *abort_flag) return false;
    }
    return false;
}

__device__ inline void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int32_t x, int32_t y,
                                   int32_t z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
        "[%2];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
        : "memory");
}

// UMMA shared-memory descriptor: K-major, 128B swizzle, 8-row groups 1024 B apart.
__device__ inline uint64_t umma_desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);          // start address
    d |= (uint64_t)1 << 16;                          // leading byte offset (unused for SW128 K-major)
    d |= (uint64_t)(1024 >> 4) << 32;                // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1 << 46;                          // descriptor version (sm_100 family)
    d |= (uint64_t)2 << 61;                          // layout: SWIZZLE_128B
    return d;
}

// instruction descriptor: kind::tf32, D = F32, A = B = TF32, both K-major, M = 128, N = 128
constexpr uint32_t tc_idesc_tf32() {
    return (1u << 4)                       // D format F32
           | (2u << 7)                     // A format TF32
           | (2u << 10)                    // B format TF32
           | ((uint32_t)(TC_BN >> 3) << 17) | ((uint32_t)(TC_BM >> 4) << 24);
}

__device__ inline void tc_mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ inline void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// one lane polls, the warp gets the result (tcgen05.ld needs the whole warp on the same path)
__device__ inline bool mbar_wait_warp(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                      uint32_t limit = TC_SPIN_LIMIT) {
    int ok = 0;
    if ((threadIdx.x & 31) == 0) ok = mbar_wait(bar, parity, abort_flag, limit) ? 1 : 0;
    return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

__device__ inline void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
#pragma unroll
    for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]);
}

template <class EPI, int FLUSH = 1, bool DF = false>
__global__ void __launch_bounds__(TC_THREADS, DF ? 1 : 2)
    k_tc_gemm_tf32(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, int64_t M,
                   int64_t N, const __grid_constant__ TcKMap ka, const __grid_constant__ TcKMap kb_map,
                   int64_t lower_div, int32_t ksplit, int32_t kchunk, EPI epi, int* err, TcFault flt) {
    // lower_div > 0: skip tiles whose rows (divided by lower_div) all lie above the diagonal
    if (lower_div > 0 && ((int64_t)blockIdx.x * TC_BM + TC_BM - 1) / lower_div < (int64_t)blockIdx.y * TC_BN) return;
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    unsigned char* base = (unsigned char*)(((uintptr_t)tc_smem_raw + 1023) & ~(uintptr_t)1023);
    float* sA = (float*)base;                                      // TC_STAGES x 16 KB
    float* sB = (float*)(base + TC_STAGES * TC_A_BYTES);           // TC_STAGES x 8 KB
    uint64_t* bars = (uint64_t*)(base + TC_STAGES * (TC_A_BYTES + TC_B_BYTES));
    uint64_t* full = bars;                   // TMA -> MMA
    uint64_t* empty = bars + TC_STAGES;      // MMA -> TMA
    uint64_t* tfull = bars + 2 * TC_STAGES;  // MMA -> accumulators (2 TMEM buffers)
    uint64_t* tfree = tfull + 2;             // accumulators -> MMA
    uint64_t* accum = tfree + 2;             // all MMAs issued so far are complete
    uint32_t* tmem_slot = (uint32_t*)(accum + 1);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
    volatile int* n_issued = abort_flag + 1;    // k blocks whose TMA loads were issued
    volatile int* n_consumed = abort_flag + 2;  // k blocks consumed by the MMA issuer

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // split-K: blockIdx.z = b * ksplit + s; split s runs K blocks [s kchunk, min(nk, (s+1) kchunk))
    const int64_t m0 = (int64_t)blockIdx.x * TC_BM, n0 = (int64_t)blockIdx.y * TC_BN;
    const int64_t b = blockIdx.z / ksplit;
    const int kb_lo = (int)(blockIdx.z - b * ksplit) * kchunk;
    const int nk_all = ka.nkp * ka.nseg;
    const int nk = (nk_all - kb_lo < kchunk) ? (nk_all - kb_lo) : kchunk;   // K blocks of this CTA

    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int t = 0; t < 2; ++t) {
            mbar_init(&tfull[t], 1);
            mbar_init(&tfree[t], 4);
        }
        mbar_init(accum, 1);
        *abort_flag = 0;
        *n_issued = 0;
        *n_consumed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TC_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // ---- TMA producer
            for (int kb = 0; kb < nk; ++kb) {
                const int s = kb % TC_STAGES;
                const uint32_t ph = (uint32_t)(kb / TC_STAGES) & 1u;
                if (kb == flt.stop_loads_at) break;   // failure injection: this block never arrives
                if (kb >= TC_STAGES && !mbar_wait(&empty[s], ph ^ 1u, abort_flag, flt.spin_limit)) {
                    *abort_flag = 1;
                    break;
                }
                if (*abort_flag) break;
                mbar_expect_tx(&full[s], TC_A_BYTES + TC_B_BYTES);
                const int kg = kb_lo + kb;
                const int sa = kg / ka.nkp, ra = kg - sa * ka.nkp;
                const int sb = kg / kb_map.nkp, rb = kg - sb * kb_map.nkp;
                tma_load_3d(sA + s * (TC_A_BYTES / 4), &mapA, &full[s], ka.koff + ra * TC_BK, (int32_t)m0,
                            ka.zsel[sa] + ka.zbatch * (int32_t)b);
                tma_load_3d(sB + s * (TC_B_BYTES / 4), &mapB, &full[s], kb_map.koff + rb * TC_BK, (int32_t)n0,
                            kb_map.zsel[sb] + kb_map.zbatch * (int32_t)b);
                *n_issued = kb + 1;
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer: each group of FLUSH K blocks accumulates alone into TMEM buffer
            // (group & 1)
            const uint32_t idesc = tc_idesc_tf32();
            for (int kb = 0; kb < nk; ++kb) {
                const int s = kb % TC_STAGES;
                const uint32_t ph = (uint32_t)(kb / TC_STAGES) & 1u;
                const int grp = kb / FLUSH, buf = grp & 1, use = grp >> 1;
                const bool first = (kb % FLUSH) == 0;
                const bool last = (kb % FLUSH) == FLUSH - 1 || kb == nk - 1;
                if (!mbar_wait(&full[s], ph, abort_flag, flt.spin_limit)) {
                    *abort_flag = 1;
                    break;
                }
                if (first && use > 0 &&
                    !mbar_wait(&tfree[buf], (uint32_t)(use - 1) & 1u, abort_flag, flt.spin_limit)) {
                    *abort_flag = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t a0 = smem_u32(sA + s * (TC_A_BYTES / 4)), b0 = smem_u32(sB + s * (TC_B_BYTES / 4));
#pragma unroll
                for (int kk = 0; kk < TC_BK / 8; ++kk) {
                    // K = 8 tf32 = 32 bytes per MMA: advance the start address inside the 128B swizzle atom
                    tc_mma_tf32(tmem + (uint32_t)(buf * TC_BN), umma_desc_sw128(a0 + kk * 32),
                                umma_desc_sw128(b0 + kk * 32), idesc, (!first || kk > 0) ? 1u : 0u);
                }
                tc_commit(&empty[s]);              // frees the stage once these MMAs have read it
                if (last) tc_commit(&tfull[buf]);  // the group's partial product is in TMEM
                *n_consumed = kb + 1;
            }
            // arrives once every MMA issued above has completed (immediately if none was issued)
            tc_commit(accum);
        }
    } else {
        // ---- accumulators: warp w reads TMEM lanes 32 (w % 4) .. + 31 = tile rows
        const int quarter = warp & 3;
        const int64_t row = m0 + quarter * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(quarter * 32) << 16);
        float acc[TC_BN];
        float lo[DF ? TC_BN : 1];
#pragma unroll
        for (int q = 0; q < TC_BN; ++q) acc[q] = 0.f;
        if constexpr (DF) {
#pragma unroll
            for (int q = 0; q < TC_BN; ++q) lo[q] = 0.f;
        }
        bool ok = true;
        const int ngrp = (nk + FLUSH - 1) / FLUSH;
        for (int grp = 0; grp < ngrp; ++grp) {
            const int buf = grp & 1, use = grp >> 1;
            if (!mbar_wait_warp(&tfull[buf], (uint32_t)use & 1u, abort_flag, flt.spin_limit)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            float scl = 1.f;
            // 2^-sexp (0 <= sexp <= 100) built from its exponent bits: exact
            if constexpr (DF) scl = __int_as_float((127 - (int)ka.sexp[(kb_lo + grp * FLUSH) / ka.nkp]) << 23);
#pragma unroll
            for (int h = 0; h < TC_BN; h += 32) {
                float v[32];
                tmem_ld32(trow + (uint32_t)(buf * TC_BN + h), v);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if constexpr (DF) {
                    // error-free TwoSum of the exactly scaled block into (acc, lo)
#pragma unroll
                    for (int q = 0; q < 32; ++q) {
                        const float x = v[q] * scl;
                        const float sm = acc[h + q] + x;
                        const float bp = sm - acc[h + q];
                        lo[h + q] += (acc[h + q] - (sm - bp)) + (x - bp);
                        acc[h + q] = sm;
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < 32; ++q) acc[h + q] += v[q];
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&tfree[buf]);
        }
        // warp-uniform decision (the epilogue functors shuffle across the warp)
        const bool failed = __shfl_sync(0xffffffffu, (!ok || *abort_flag) ? 1 : 0, 0) != 0;
        if (failed) {
            if (lane == 0) *abort_flag = 1;
        } else if (nk > 0) {
            if constexpr (DF) {
#pragma unroll
                for (int h = 0; h < TC_BN; h += 32) {
                    double d[32];
#pragma unroll
                    for (int q = 0; q < 32; ++q) d[q] = (double)acc[h + q] + (double)lo[h + q];
                    epi((int64_t)blockIdx.z, row, n0 + h, d, M, N);
                }
            } else {
                epi((int64_t)blockIdx.z, row, n0, acc, M, N);
                epi((int64_t)blockIdx.z, row, n0 + 32, acc + 32, M, N);
            }
        }
    }
    __syncthreads();
    if (*abort_flag && threadIdx.x == 0) {
        atomicExch(err, 1);
        // drain: the MMAs in flight (accum) and the TMA loads issued but not consumed
        mbar_wait(accum, 0, nullptr, flt.spin_limit);
        for (int kb = *n_consumed; kb < *n_issued; ++kb)
            mbar_wait(&full[kb % TC_STAGES], (uint32_t)(kb / TC_STAGES) & 1u, nullptr, flt.spin_limit);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS));
    }
}

// Number of K splits actually launched for nk K blocks when `want` are asked for: every split
// gets ceil(nk / want) blocks, the last one the rest, and none is empty.
inline int tc_ksplit_count(int64_t nk, int want) {
    if (want <= 1 || nk <= 1) return 1;
    const int64_t chunk = (nk + want - 1) / want;
    return (int)((nk + chunk - 1) / chunk);
}

// Host launcher: D tiles for b < batch; the epilogue gets (z, row, col0, v[32], M, N) and must
// bounds-check row < M and col0 + q < N itself; z = b * ks + s, where ks = tc_ksplit_count(nk,
// ksplit) splits of the K range each produce a partial product (ks = 1 without split-K: z = b).
// Both K maps must cover the same number of K blocks.  Every TMA x coordinate (koff + 32 j) is
// a multiple of 4 floats (16 bytes).
template <class EPI, int FLUSH = 1, bool DF = false>
int tc_gemm_tf32_mapped(cudaStream_t st, const TcOperand& A, const TcKMap& ka, const TcOperand& B, const TcKMap& kb,
                        int64_t batch, int64_t lower_div, const EPI& epi, int* err, int ksplit = 1,
                        TcFault flt = TcFault{}) {
    if (A.rows <= 0 || B.rows <= 0 || batch <= 0) return 0;
    if (FLUSH > 1 && (ksplit != 1 || ka.nkp % FLUSH || kb.nkp % FLUSH)) {
        set_error(FORGE_ERR_ARG, "tc_gemm: exact-block mode needs whole flush groups per segment and no K split");
        return FORGE_ERR_ARG;
    }
    if ((A.ld % 4) || (B.ld % 4) || (A.batch_stride % 4) || (B.batch_stride % 4) || (ka.koff % 4) || (kb.koff % 4) ||
        ((uintptr_t)A.ptr % 16) || ((uintptr_t)B.ptr % 16)) {
        set_error(FORGE_ERR_ARG, "tc_gemm: operands must be 16-byte aligned with pitches multiple of 4 floats");
        return FORGE_ERR_ARG;
    }
    if (ka.nkp * ka.nseg != kb.nkp * kb.nseg || ka.nseg < 1 || ka.nseg > TC_MAXSEG || kb.nseg < 1 ||
        kb.nseg > TC_MAXSEG) {
        set_error(FORGE_ERR_ARG, "tc_gemm: inconsistent K maps");
        return FORGE_ERR_ARG;
    }
    CUtensorMap ma, mb;
    FORGE_TRY(tc_make_tmap(&ma, A, batch, TC_BM));
    FORGE_TRY(tc_make_tmap(&mb, B, batch, TC_BN));
    static bool attr_set = false;
    if (!attr_set) {
        FORGE_CUDA(cudaFuncSetAttribute(k_tc_gemm_tf32<EPI, FLUSH, DF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        TC_SMEM));
        attr_set = true;
    }
    const int64_t nk = (int64_t)ka.nkp * ka.nseg;
    const int ks = tc_ksplit_count(nk, ksplit);
    const int32_t kchunk = (int32_t)((nk + ks - 1) / ks);
    if (batch * ks > 65535) {
        set_error(FORGE_ERR_ARG, "tc_gemm: batch x K splits exceeds the grid's z extent");
        return FORGE_ERR_ARG;
    }
    dim3 grd((unsigned)((A.rows + TC_BM - 1) / TC_BM), (unsigned)((B.rows + TC_BN - 1) / TC_BN),
             (unsigned)(batch * ks));
    k_tc_gemm_tf32<EPI, FLUSH, DF><<<grd, TC_THREADS, TC_SMEM, st>>>(ma, mb, A.rows, B.rows, ka, kb, lower_div, ks,
                                                                     kchunk, epi, err, flt);
    FORGE_LAUNCH_CHECK();
    return 0;
}

// Plain form: row-major A (M x K) and B (N x K), batch in the 3rd dimension.
template <class EPI>
int tc_gemm_tf32(cudaStream_t st, const TcOperand& A, const TcOperand& B, int64_t K, int64_t batch, const EPI& epi,
                 int* err, int64_t lower_div = 0, TcFault flt = TcFault{}) {
    TcOperand a = A, bb = B;
    a.cols = K;
    bb.cols = K;
    a.nplanes = batch;
    bb.nplanes = batch;
    return tc_gemm_tf32_mapped(st, a, tc_kmap_plain(K), bb, tc_kmap_plain(K), batch, lower_div, epi, err, 1, flt);
}

}  // namespace forge
