/*
 * Learned initial guess: the kernels of a small MLP (BF16 tensor-core GEMMs
 * with FP32 accumulation, forward and backward, Adam) and of the POD
 * subspace it predicts in (projection of states onto the basis, expansion of
 * predicted coefficients into a correction vector).
 *
 * The network maps the POD projections of the last four states and the
 * pulse factors f_a(t) to the POD coefficients of the part of the next state
 * that linear extrapolation misses (x_{n+1} - 2 x_n + x_{n-1}); the mixed
 * precision step then starts from x_n + (x_n - x_{n-1}) + U c.  Everything
 * here works on device pointers handed in by the host; nothing allocates.
 *
 * Tensor-core path: tcgen05.mma (BF16 in, FP32 accumulate in tensor
 * memory) from shared-memory tiles, one elected thread issuing, completion
 * tracked by mbarriers.  The GEMMs of this network are a few MFLOP per step
 * (M = pulses, N = 256) and ~1 GFLOP per training epoch, far from any
 * roofline; the kernels favour exact, checkable arithmetic over peak
 * throughput.
 */
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <math.h>

#include "gade.h"
#include "gade_learned.h"

extern "C" int gade_set_error(int code, const char *msg);

static int lfail(int code, const char *what, cudaError_t e)
{
    char buf[512];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return gade_set_error(code, buf);
}

#define LCK(what)                                                                    \
    do {                                                                             \
        cudaError_t e_ = cudaGetLastError();                                         \
        if (e_ != cudaSuccess) return lfail(GADE_ERR_CUDA, what, e_);                \
    } while (0)

typedef __nv_bfloat16 bf16;

/* ------------------------------------------------------------------ */
/* GEMM: C = epi(A B + bias) on the 5th-generation tensor cores         */
/* ------------------------------------------------------------------ */
/* A(i,k) = A[i*sa0 + k*sa1], B(k,j) = B[k*sb0 + j*sb1] (any transposition),
 * FP32 accumulation.  Epilogue: + bias[j]; times (mask(i,j) > 0) when a
 * mask is given (ReLU backward); ReLU when act = 1; FP32 result to C and/or
 * a BF16 copy to C16.
 *
 * One CTA computes a 128 x 64 tile of C with tcgen05.mma (kind::f16, BF16
 * A and B, FP32 accumulator in tensor memory, M = 128, N = 64, K = 16 per
 * instruction), 64-wide K blocks staged in shared memory in the no-swizzle
 * canonical layouts of 8 x 16-byte core matrices: element (r, k) of an
 * operand tile (r along M or N, k along K) sits at
 *     (r/8)*SBO + (k/8)*LBO + (r%8)*16 + (k%8)*2          (K-major)
 *     (r/8)*SBO + (k/8)*LBO + (k%8)*16 + (r%8)*2          (M/N-major)
 * bytes, LBO and SBO in the shared-memory descriptor of each MMA.
 *
 * k_gemm_tma (operands 16-byte aligned with 16-byte row strides): one
 * thread fills a GST-deep ring of stages with 2-D tensor copies
 * (cp.async.bulk.tensor, boxes 16 bytes wide so that each copy lands as a
 * column of core matrices; out-of-range rows and columns arrive as zeros),
 * one thread issues the MMAs of a stage once its mbarrier has seen all
 * bytes and frees the stage with tcgen05.commit on the stage's empty
 * mbarrier, and all four warps read the accumulator back with tcgen05.ld
 * (warp w owns TMEM lanes 32w..32w+31 = tile rows) for the epilogue.  An
 * operand contiguous along K is staged K-major; one contiguous along M or N
 * is staged M/N-major with the descriptor's transpose bit, so no operand is
 * transposed by the SMs.
 *
 * k_gemm_ld (any strides): the four warps stage each K block with plain
 * loads into two K-major buffers while the tensor core multiplies the
 * other.
 *
 * Every mbarrier wait is bounded: on a timeout the CTA records it in the
 * learned-kernel status word, waits (bounded) for its copies and MMAs in
 * flight, frees its tensor memory and returns without writing its tile. */
#define GTM 128
#define GTN 64
#define GTK 64
#define GST 4                            /* stages of the tensor-copy ring */
#define GSTAGE ((GTM + GTN) * GTK * 2)   /* bytes of one stage: A then B */
#define GSPIN_DEFAULT (1u << 24)
#define GDRAIN (1u << 24)

static __device__ unsigned g_learned_err;   /* bit 0: a tensor-core wait ran out */
static unsigned g_gemm_spin = GSPIN_DEFAULT; /* waits before a CTA gives up */
static int g_gemm_path = 0;                  /* 0 automatic, 1 plain loads */
static int g_gemm_withhold = 0;              /* 1: the copy thread issues nothing */

__device__ __forceinline__ unsigned l_smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ bool l_try_wait(uint64_t *bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(l_smem_u32(bar)), "r"(parity) : "memory");
    return ok != 0;
}
/* bounded wait; false when it ran out (or another thread of the CTA gave up) */
__device__ __forceinline__ bool l_wait(uint64_t *bar, unsigned parity, unsigned limit, volatile int *fail)
{
    for (unsigned spins = 0; !l_try_wait(bar, parity);)
        if (++spins > limit || (fail && *fail)) return false;
    return true;
}
/* shared-memory matrix descriptor: start address, leading (K) and stride
   (8-row group) byte offsets, the tcgen05 descriptor version, no swizzle */
__device__ __forceinline__ uint64_t l_sdesc(unsigned addr, unsigned lbo, unsigned sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}
/* instruction descriptor: FP32 accumulator, BF16 A and B, A/B M/N-major when
   a_mn/b_mn (transpose bits), N and M of the tile */
__device__ __forceinline__ unsigned l_idesc(bool a_mn, bool b_mn)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
           ((unsigned)(GTN >> 3) << 17) | ((unsigned)(GTM >> 4) << 24);
}
__device__ __forceinline__ void l_mma(unsigned tmem, uint64_t ad, uint64_t bd, unsigned idesc, unsigned acc)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                 "l"(ad), "l"(bd), "r"(idesc), "r"(acc) : "memory");
}
__device__ __forceinline__ void l_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     l_smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void l_tmem_alloc(unsigned *dst)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(l_smem_u32(dst)),
                 "r"(GTN) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void l_tmem_free(unsigned tmem)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(GTN) : "memory");
}

/* accumulator rows -> epilogue -> C / C16; warp w reads TMEM lanes 32w.. */
__device__ __forceinline__ void l_epilogue(unsigned tmem, bool have_acc, int M, int N, int i0, int j0,
                                           const float *__restrict__ bias, const float *__restrict__ mask,
                                           long long ldm, int act, float *__restrict__ C, long long ldc,
                                           bf16 *__restrict__ C16, long long ldc16)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = i0 + warp * 32 + lane;
    for (int c0 = 0; c0 < GTN; c0 += 16) {
        if (j0 + c0 >= N) break;               /* warp-uniform */
        unsigned v[16];
        const unsigned taddr = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)c0;
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
                     "%14,%15}, [%16];"
                     : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                       "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                       "=r"(v[14]), "=r"(v[15])
                     : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (i >= M) continue;
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int j = j0 + c0 + q;
            if (j >= N) continue;
            float val = have_acc ? __uint_as_float(v[q]) : 0.f;   /* K = 0: no MMA wrote TMEM */
            if (bias) val += bias[j];
            if (mask && !(mask[i * ldm + j] > 0.f)) val = 0.f;
            if (act == 1) val = val > 0.f ? val : 0.f;
            if (C) C[i * ldc + j] = val;
            if (C16) C16[i * ldc16 + j] = __float2bfloat16(val);
        }
    }
}

__device__ __forceinline__ void l_tma2d(unsigned dst, const CUtensorMap *map, int x, int y, uint64_t *bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
                 "%3}], [%4];" ::"r"(dst),
                 "l"((uint64_t)map), "r"(x), "r"(y), "r"(l_smem_u32(bar)) : "memory");
}

/* A_MN: A staged M-major (A contiguous along M), else K-major; B_MN likewise
   along N.  Tensor maps: K-major operand {K, rows}, box {8, rows of the
   tile}, one copy per 8-wide K slice (LBO = rows x 16 B, SBO = 128 B);
   M/N-major operand {rows, K}, box {8, 64}, one copy per 8 rows (LBO =
   128 B, SBO = 1 KB).  Every x coordinate is a multiple of 8 elements. */
template <bool A_MN, bool B_MN>
__global__ void __launch_bounds__(128) k_gemm_tma(const __grid_constant__ CUtensorMap mapA,
                                                  const __grid_constant__ CUtensorMap mapB, int M, int N, int K,
                                                  const float *__restrict__ bias, const float *__restrict__ mask,
                                                  long long ldm, int act, float *__restrict__ C, long long ldc,
                                                  bf16 *__restrict__ C16, long long ldc16, unsigned spin_limit,
                                                  int withhold)
{
    extern __shared__ __align__(1024) unsigned char gsm[];   /* [GST][A 128x64 | B 64x64] */
    __shared__ __align__(8) uint64_t full[GST], empty[GST];
    __shared__ unsigned tmem_base;
    __shared__ int s_copied, s_issued;          /* K blocks copied / multiplied */
    __shared__ volatile int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int i0 = blockIdx.y * GTM, j0 = blockIdx.x * GTN;
    constexpr unsigned A_LBO = A_MN ? 128 : GTM * 16, A_SBO = A_MN ? 1024 : 128;
    constexpr unsigned B_LBO = B_MN ? 128 : GTN * 16, B_SBO = B_MN ? 1024 : 128;
    if (warp == 0) l_tmem_alloc(&tmem_base);
    if (tid == 0) {
        for (int b = 0; b < GST; b++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(l_smem_u32(&full[b])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(l_smem_u32(&empty[b])) : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_copied = 0;
        s_issued = 0;
        s_fail = 0;
    }
    if (tid == 32) {
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&mapA) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&mapB) : "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = tmem_base;
    const int nkb = (K + GTK - 1) / GTK;
    const unsigned gbase = l_smem_u32(gsm);

    if (tid == 0) {                            /* copy thread */
        for (int kb = 0; kb < nkb && !withhold; kb++) {
            const int st = kb % GST, k0 = kb * GTK;
            if (kb >= GST && !l_wait(&empty[st], ((kb / GST) - 1) & 1, spin_limit, &s_fail)) {
                s_fail = 1;
                break;
            }
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(l_smem_u32(&full[st])),
                         "r"(GSTAGE) : "memory");
            const unsigned As = gbase + st * GSTAGE, Bs = As + GTM * GTK * 2;
            if (A_MN)
                for (int g = 0; g < GTM / 8; g++) l_tma2d(As + g * 1024, &mapA, i0 + 8 * g, k0, &full[st]);
            else
                for (int q = 0; q < GTK / 8; q++) l_tma2d(As + q * GTM * 16, &mapA, k0 + 8 * q, i0, &full[st]);
            if (B_MN)
                for (int g = 0; g < GTN / 8; g++) l_tma2d(Bs + g * 1024, &mapB, j0 + 8 * g, k0, &full[st]);
            else
                for (int q = 0; q < GTK / 8; q++) l_tma2d(Bs + q * GTN * 16, &mapB, k0 + 8 * q, j0, &full[st]);
            s_copied = kb + 1;
        }
    } else if (tid == 32) {                    /* MMA thread */
        const unsigned idesc = l_idesc(A_MN, B_MN);
        for (int kb = 0; kb < nkb; kb++) {
            const int st = kb % GST;
            if (!l_wait(&full[st], (kb / GST) & 1, spin_limit, &s_fail)) {
                s_fail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const unsigned As = gbase + st * GSTAGE, Bs = As + GTM * GTK * 2;
#pragma unroll
            for (int kk = 0; kk < GTK / 16; kk++)
                l_mma(tmem, l_sdesc(As + kk * 2 * A_LBO, A_LBO, A_SBO), l_sdesc(Bs + kk * 2 * B_LBO, B_LBO, B_SBO),
                      idesc, (kb > 0 || kk > 0) ? 1u : 0u);
            l_commit(&empty[st]);              /* frees the stage; the last one also marks the end */
            s_issued = kb + 1;
        }
    }
    __syncthreads();
    /* every thread: the last commit covers every MMA issued before it */
    bool ok = !s_fail;
    if (ok && nkb > 0) ok = l_wait(&empty[(nkb - 1) % GST], ((nkb - 1) / GST) & 1, spin_limit, nullptr);
    ok = !__syncthreads_or(!ok);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
        l_epilogue(tmem, nkb > 0, M, N, i0, j0, bias, mask, ldm, act, C, ldc, C16, ldc16);
    } else if (tid == 0) {
        atomicOr(&g_learned_err, 1u);
        /* copies in flight: the stages copied and not yet seen complete */
        for (int kb = s_copied - GST > 0 ? s_copied - GST : 0; kb < s_copied; kb++)
            l_wait(&full[kb % GST], (kb / GST) & 1, GDRAIN, nullptr);
        if (s_issued > 0) l_wait(&empty[(s_issued - 1) % GST], ((s_issued - 1) / GST) & 1, GDRAIN, nullptr);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) l_tmem_free(tmem);
}

__global__ void __launch_bounds__(128) k_gemm_ld(int M, int N, int K, const bf16 *__restrict__ A, long long sa0,
                                                 long long sa1, const bf16 *__restrict__ B, long long sb0,
                                                 long long sb1, const float *__restrict__ bias,
                                                 const float *__restrict__ mask, long long ldm, int act,
                                                 float *__restrict__ C, long long ldc, bf16 *__restrict__ C16,
                                                 long long ldc16, unsigned spin_limit)
{
    extern __shared__ __align__(1024) unsigned char gsm[];   /* [2][A 128x64 | B 64x64] */
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ unsigned tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int i0 = blockIdx.y * GTM, j0 = blockIdx.x * GTN;
    constexpr unsigned LBO = 128, SBO = (GTK / 8) * 128;   /* K-major, 8 core matrices per row group */
    if (warp == 0) l_tmem_alloc(&tmem_base);
    if (tid == 0) {
        for (int b = 0; b < 2; b++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(l_smem_u32(&bar[b])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = tmem_base;
    const unsigned idesc = l_idesc(false, false);
    const bf16 zero = __float2bfloat16(0.f);
    const int nkb = (K + GTK - 1) / GTK;
    bool ok = true;
    int issued = 0;                            /* K blocks whose MMAs were committed */
    for (int kb = 0; kb < nkb; kb++) {
        const int b = kb & 1, k0 = kb * GTK;
        unsigned char *As = gsm + b * GSTAGE, *Bs = As + GTM * GTK * 2;
        if (kb >= 2) ok = l_wait(&bar[b], ((kb - 2) >> 1) & 1, spin_limit, nullptr);   /* block kb-2 done */
        if (__syncthreads_or(!ok)) { ok = false; break; }
        for (int e = tid; e < GTM * GTK; e += 128) {
            const int r = e / GTK, k = e % GTK;
            const int gi = i0 + r, gk = k0 + k;
            *(bf16 *)(As + (r >> 3) * SBO + (k >> 3) * LBO + (r & 7) * 16 + (k & 7) * 2) =
                (gi < M && gk < K) ? A[gi * sa0 + gk * sa1] : zero;
        }
        for (int e = tid; e < GTN * GTK; e += 128) {
            const int c = e / GTK, k = e % GTK;
            const int gj = j0 + c, gk = k0 + k;
            *(bf16 *)(Bs + (c >> 3) * SBO + (k >> 3) * LBO + (c & 7) * 16 + (k & 7) * 2) =
                (gj < N && gk < K) ? B[gk * sb0 + gj * sb1] : zero;
        }
        /* the generic-proxy stores become visible to the tensor core */
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (tid == 0) {
            for (int kk = 0; kk < GTK / 16; kk++)
                l_mma(tmem, l_sdesc(l_smem_u32(As) + kk * 2 * LBO, LBO, SBO),
                      l_sdesc(l_smem_u32(Bs) + kk * 2 * LBO, LBO, SBO), idesc, (kb > 0 || kk > 0) ? 1u : 0u);
            l_commit(&bar[b]);
        }
        issued = kb + 1;
    }
    /* the last commit covers every MMA issued before it */
    if (ok && issued > 0) ok = l_wait(&bar[(issued - 1) & 1], ((issued - 1) >> 1) & 1, spin_limit, nullptr);
    ok = !__syncthreads_or(!ok);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
        l_epilogue(tmem, issued > 0, M, N, i0, j0, bias, mask, ldm, act, C, ldc, C16, ldc16);
    } else if (tid == 0) {
        atomicOr(&g_learned_err, 1u);
        if (issued > 0) l_wait(&bar[(issued - 1) & 1], ((issued - 1) >> 1) & 1, GDRAIN, nullptr);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) l_tmem_free(tmem);
}

/* cuTensorMapEncodeTiled through the runtime's driver entry point (no link
   against the driver library) */
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
        cudaGetLastError();
    }
    return fn;
}

/* 2-D BF16 map of a (rows x inner) operand with row stride ld elements and
   box {8, box_rows}; false when the layout does not allow tensor copies */
static bool encode_operand(CUtensorMap *map, const void *base, long long inner, long long rows, long long ld,
                           int box_rows)
{
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc || ((uintptr_t)base & 15) || inner <= 0 || rows <= 0 || inner > (1ll << 32) || rows > (1ll << 32))
        return false;
    long long stride = ld * 2;
    if (rows == 1 && stride < inner * 2) stride = (inner * 2 + 15) / 16 * 16;   /* unused for one row */
    if ((stride & 15) || stride < inner * 2 || stride >= (1ll << 40)) return false;
    cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)stride};
    cuuint32_t box[2] = {8, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <bool A_MN, bool B_MN>
static cudaError_t launch_gemm_tma(dim3 grid, cudaStream_t st, const CUtensorMap &ma, const CUtensorMap &mb, int M,
                                   int N, int K, const float *bias, const float *mask, long long ldm, int act,
                                   float *C, long long ldc, bf16 *C16, long long ldc16)
{
    static unsigned long long smem_set = 0;   /* per device: GST x 24 KB is above the 48 KB default */
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev >= 64 || !(smem_set >> dev & 1ull)) {
        e = cudaFuncSetAttribute(k_gemm_tma<A_MN, B_MN>, cudaFuncAttributeMaxDynamicSharedMemorySize, GST * GSTAGE);
        if (e != cudaSuccess) return e;
        if (dev < 64) smem_set |= 1ull << dev;
    }
    k_gemm_tma<A_MN, B_MN><<<grid, 128, GST * GSTAGE, st>>>(ma, mb, M, N, K, bias, mask, ldm, act, C, ldc, C16,
                                                           ldc16, g_gemm_spin, g_gemm_withhold);
    return cudaGetLastError();
}

extern "C" int gade_gemm_bf16(int32_t M, int32_t N, int32_t K, const void *A, int64_t sa0, int64_t sa1,
                              const void *B, int64_t sb0, int64_t sb1, const float *bias, const float *mask,
                              int64_t ldm, int32_t act, float *C, int64_t ldc, void *C16, int64_t ldc16,
                              void *stream)
{
    if (M < 0 || N < 0 || K < 0 || !A || !B || (!C && !C16) || (act != 0 && act != 1))
        return gade_set_error(GADE_ERR_ARG, "gade_gemm_bf16: bad argument");
    if (M == 0 || N == 0) return GADE_OK;
    cudaStream_t st = (cudaStream_t)stream;
    dim3 grid((N + GTN - 1) / GTN, (M + GTM - 1) / GTM);
    if (g_gemm_path == 0 && K > 0) {
        /* A contiguous along K (sa1 = 1) is staged K-major, along M (sa0 = 1)
           M-major; B contiguous along K (sb0 = 1) K-major, along N N-major */
        CUtensorMap ma, mb;
        const bool a_k = sa1 == 1, b_k = sb0 == 1;
        const bool a_ok = a_k ? encode_operand(&ma, A, K, M, sa0, GTM)
                              : (sa0 == 1 && encode_operand(&ma, A, M, K, sa1, GTK));
        const bool b_ok = b_k ? encode_operand(&mb, B, K, N, sb1, GTN)
                              : (sb1 == 1 && encode_operand(&mb, B, N, K, sb0, GTK));
        if (a_ok && b_ok) {
            cudaError_t e;
            if (!a_k && !b_k) e = launch_gemm_tma<true, true>(grid, st, ma, mb, M, N, K, bias, mask, ldm, act, C,
                                                              ldc, (bf16 *)C16, ldc16);
            else if (!a_k) e = launch_gemm_tma<true, false>(grid, st, ma, mb, M, N, K, bias, mask, ldm, act, C, ldc,
                                                            (bf16 *)C16, ldc16);
            else if (!b_k) e = launch_gemm_tma<false, true>(grid, st, ma, mb, M, N, K, bias, mask, ldm, act, C, ldc,
                                                            (bf16 *)C16, ldc16);
            else e = launch_gemm_tma<false, false>(grid, st, ma, mb, M, N, K, bias, mask, ldm, act, C, ldc,
                                                   (bf16 *)C16, ldc16);
            if (e != cudaSuccess) return lfail(GADE_ERR_CUDA, "gade_gemm_bf16", e);
            return GADE_OK;
        }
    }
    static unsigned long long smem_set = 0;   /* per device: 2 x 24 KB is above the 48 KB default */
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return lfail(GADE_ERR_CUDA, "gade_gemm_bf16", e);
    if (dev >= 64 || !(smem_set >> dev & 1ull)) {
        e = cudaFuncSetAttribute(k_gemm_ld, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * GSTAGE);
        if (e != cudaSuccess) return lfail(GADE_ERR_CUDA, "gade_gemm_bf16", e);
        if (dev < 64) smem_set |= 1ull << dev;
    }
    k_gemm_ld<<<grid, 128, 2 * GSTAGE, st>>>(M, N, K, (const bf16 *)A, sa0, sa1, (const bf16 *)B, sb0, sb1, bias,
                                             mask, ldm, act, C, ldc, (bf16 *)C16, ldc16, g_gemm_spin);
    LCK("gade_gemm_bf16");
    return GADE_OK;
}

extern "C" int gade_gemm_bf16_path(int32_t M, int32_t N, int32_t K, const void *A, int64_t sa0, int64_t sa1,
                                   const void *B, int64_t sb0, int64_t sb1)
{
    if (g_gemm_path != 0 || K <= 0 || M <= 0 || N <= 0) return 0;
    CUtensorMap ma, mb;
    const bool a_ok = sa1 == 1 ? encode_operand(&ma, A, K, M, sa0, GTM)
                               : (sa0 == 1 && encode_operand(&ma, A, M, K, sa1, GTK));
    const bool b_ok = sb0 == 1 ? encode_operand(&mb, B, K, N, sb1, GTN)
                               : (sb1 == 1 && encode_operand(&mb, B, N, K, sb0, GTK));
    return a_ok && b_ok ? 1 : 0;
}

extern "C" int gade_learned_set_gemm_options(int32_t path, uint32_t wait_limit, int32_t withhold_copies)
{
    if (path < 0 || path > 1 || withhold_copies < 0 || withhold_copies > 1)
        return gade_set_error(GADE_ERR_ARG, "gade_learned_set_gemm_options: bad argument");
    g_gemm_path = path;
    g_gemm_spin = wait_limit ? wait_limit : GSPIN_DEFAULT;
    g_gemm_withhold = withhold_copies;
    return GADE_OK;
}

extern "C" int gade_learned_status(int32_t *flags)
{
    if (!flags) return gade_set_error(GADE_ERR_ARG, "gade_learned_status: NULL argument");
    unsigned v = 0, z = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_learned_err, sizeof(v));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_learned_err, &z, sizeof(z));
    if (e != cudaSuccess) return lfail(GADE_ERR_CUDA, "gade_learned_status", e);
    *flags = (int32_t)v;
    return GADE_OK;
}

/* ------------------------------------------------------------------ */
/* loss, bias gradient, Adam, conversions                              */
/* ------------------------------------------------------------------ */
/* mean squared error over M x N: grad = 2 (out - target) / (M N) (FP32 and
 * BF16), per-row partial sums of the squared error into rowloss[M] */
__global__ void k_mse(int M, int N, const float *__restrict__ out, const float *__restrict__ target,
                      float *__restrict__ grad, bf16 *__restrict__ grad16, double *__restrict__ rowloss)
{
    const int i = blockIdx.x;
    if (i >= M) return;
    __shared__ double sh[256];
    double s = 0;
    const float scale = 2.0f / ((float)M * (float)N);
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        const float d = out[(size_t)i * N + j] - target[(size_t)i * N + j];
        const float g = scale * d;
        if (grad) grad[(size_t)i * N + j] = g;
        grad16[(size_t)i * N + j] = __float2bfloat16(g);
        s += (double)d * d;
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) rowloss[i] = sh[0];
}

extern "C" int gade_mse_grad(int32_t M, int32_t N, const float *out, const float *target, float *grad, void *grad16,
                             double *rowloss, void *stream)
{
    if (M <= 0 || N <= 0 || !out || !target || !grad16 || !rowloss)
        return gade_set_error(GADE_ERR_ARG, "gade_mse_grad: bad argument");
    k_mse<<<M, 256, 0, (cudaStream_t)stream>>>(M, N, out, target, grad, (bf16 *)grad16, rowloss);
    LCK("gade_mse_grad");
    return GADE_OK;
}

/* db[j] = sum_i G(i, j) in fixed order */
__global__ void k_colsum(int M, int N, const float *__restrict__ G, long long ldg, float *__restrict__ db)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    float s = 0.f;
    for (int i = 0; i < M; i++) s += G[(size_t)i * ldg + j];
    db[j] = s;
}

extern "C" int gade_colsum(int32_t M, int32_t N, const float *G, int64_t ldg, float *db, void *stream)
{
    if (M < 0 || N <= 0 || !G || !db) return gade_set_error(GADE_ERR_ARG, "gade_colsum: bad argument");
    k_colsum<<<(N + 255) / 256, 256, 0, (cudaStream_t)stream>>>(M, N, G, ldg, db);
    LCK("gade_colsum");
    return GADE_OK;
}

/* Adam on FP32 master weights (Kingma & Ba 2015); refreshes the BF16 copy */
__global__ void k_adam(long long n, float *__restrict__ w, bf16 *__restrict__ w16, const float *__restrict__ g,
                       float *__restrict__ m, float *__restrict__ v, float lr, float b1, float b2, float eps,
                       float c1, float c2)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        if (w16) w16[i] = __float2bfloat16(wi);
    }
}

extern "C" int gade_adam(int64_t n, float *w, void *w16, const float *g, float *m, float *v, float lr, float beta1,
                         float beta2, float eps, int32_t step, void *stream)
{
    if (n <= 0 || !w || !g || !m || !v || step < 1) return gade_set_error(GADE_ERR_ARG, "gade_adam: bad argument");
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    int grid = (int)((n + 255) / 256);
    if (grid > 4096) grid = 4096;
    k_adam<<<grid, 256, 0, (cudaStream_t)stream>>>(n, w, (bf16 *)w16, g, m, v, lr, beta1, beta2, eps, c1, c2);
    LCK("gade_adam");
    return GADE_OK;
}

__global__ void k_to_bf16(long long n, const float *__restrict__ x, bf16 *__restrict__ y)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = __float2bfloat16(x[i]);
}

extern "C" int gade_to_bf16(int64_t n, const float *x, void *y, void *stream)
{
    if (n < 0 || !x || !y) return gade_set_error(GADE_ERR_ARG, "gade_to_bf16: bad argument");
    if (n == 0) return GADE_OK;
    int grid = (int)((n + 255) / 256);
    if (grid > 4096) grid = 4096;
    k_to_bf16<<<grid, 256, 0, (cudaStream_t)stream>>>(n, x, (bf16 *)y);
    LCK("gade_to_bf16");
    return GADE_OK;
}

/* ------------------------------------------------------------------ */
/* POD subspace                                                        */
/* ------------------------------------------------------------------ */
/* coef[p][r] = sum_i conj(U[r][i]) x_p[i]: U complex64 [R][n], x complex128
 * [npulse][n] (stride ldx), FP64 accumulation.  Stage 1: grid (pulse,
 * chunk); every block stages its x slice in shared memory and 8 warps take
 * the basis rows; partials [chunk][p][r].  Stage 2 sums chunks in order. */
#define PJ_L 1024
/* FP64 -> FP32 by bit operations, without the conversion instruction (which
   runs at the FP64 rate on this GPU): sign, rebiased exponent and the top 23
   mantissa bits (truncation, relative error < 2^-23); magnitudes below the
   FP32 normal range give 0, above it infinity, NaN stays NaN. */
__device__ __forceinline__ float l_f32_bits(double v)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const int e11 = (int)((b >> 52) & 0x7FF);
    const unsigned mant = (unsigned)((b >> 29) & 0x7FFFFF);
    if (e11 == 0x7FF) return __uint_as_float(sign | 0x7F800000u | (b & 0xFFFFFFFFFFFFFull ? 0x400000u : 0u));
    const int e8 = e11 - 1023 + 127;
    if (e8 <= 0) return __uint_as_float(sign);
    if (e8 >= 255) return __uint_as_float(sign | 0x7F800000u);
    return __uint_as_float(sign | ((unsigned)e8 << 23) | mant);
}

/* partial projections of one 1024-element chunk of one pulse's state: the
   network's BF16 inputs need no more than FP32 products and per-chunk FP32
   sums (relative error ~1e-7); chunks are added in FP64 in a fixed order */
__global__ void __launch_bounds__(256) k_pod_partial(int n, int R, const float2 *__restrict__ U,
                                                     const double2 *__restrict__ x, long long ldx,
                                                     double2 *__restrict__ part, int npulse)
{
    __shared__ float2 xs[PJ_L];
    const int p = blockIdx.x, ch = blockIdx.y;
    const int i0 = ch * PJ_L;
    const int len = n - i0 < PJ_L ? n - i0 : PJ_L;
    const double2 *xp = x + (size_t)p * ldx + i0;
    for (int e = threadIdx.x; e < len; e += 256) {
        const double2 v = xp[e];
        xs[e] = make_float2(l_f32_bits(v.x), l_f32_bits(v.y));
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int r = warp; r < R; r += 8) {
        const float2 *u = U + (size_t)r * n + i0;
        float sr = 0.f, si = 0.f;
        for (int e = lane; e < len; e += 32) {
            const float2 uv = u[e];
            const float2 xv = xs[e];
            sr = fmaf(uv.x, xv.x, fmaf(uv.y, xv.y, sr));      /* conj(u) x */
            si = fmaf(uv.x, xv.y, fmaf(-uv.y, xv.x, si));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sr += __shfl_xor_sync(0xffffffffu, sr, o);
            si += __shfl_xor_sync(0xffffffffu, si, o);
        }
        if (lane == 0) part[((size_t)ch * npulse + p) * R + r] = make_double2(sr, si);
    }
}

/* the same partial projections with FP64 products and sums (training
   targets are second differences of projections, which cancel) */
__global__ void __launch_bounds__(256) k_pod_partial64(int n, int R, const float2 *__restrict__ U,
                                                       const double2 *__restrict__ x, long long ldx,
                                                       double2 *__restrict__ part, int npulse)
{
    __shared__ double2 xs[PJ_L];
    const int p = blockIdx.x, ch = blockIdx.y;
    const int i0 = ch * PJ_L;
    const int len = n - i0 < PJ_L ? n - i0 : PJ_L;
    const double2 *xp = x + (size_t)p * ldx + i0;
    for (int e = threadIdx.x; e < len; e += 256) xs[e] = xp[e];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int r = warp; r < R; r += 8) {
        const float2 *u = U + (size_t)r * n + i0;
        double sr = 0, si = 0;
        for (int e = lane; e < len; e += 32) {
            const float2 uv = u[e];
            const double2 xv = xs[e];
            sr += (double)uv.x * xv.x + (double)uv.y * xv.y;
            si += (double)uv.x * xv.y - (double)uv.y * xv.x;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sr += __shfl_xor_sync(0xffffffffu, sr, o);
            si += __shfl_xor_sync(0xffffffffu, si, o);
        }
        if (lane == 0) part[((size_t)ch * npulse + p) * R + r] = make_double2(sr, si);
    }
}

__global__ void k_pod_sum(int nch, int npulse, int R, const double2 *__restrict__ part, double2 *__restrict__ coef)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npulse * R) return;
    double sr = 0, si = 0;
    for (int c = 0; c < nch; c++) {
        const double2 v = part[(size_t)c * npulse * R + t];
        sr += v.x; si += v.y;
    }
    coef[t] = make_double2(sr, si);
}

static int pod_project(bool fp64, int64_t n, int32_t R, const void *U, const void *x, int64_t ldx, int32_t npulse,
                       void *coef, void *scratch, int64_t scratch_bytes, void *stream)
{
    if (n <= 0 || n > (1ll << 31) - 1 || R <= 0 || npulse <= 0 || !U || !x || !coef || !scratch)
        return gade_set_error(GADE_ERR_ARG, "gade_pod_project: bad argument");
    const int nch = (int)((n + PJ_L - 1) / PJ_L);
    const int64_t need = (int64_t)nch * npulse * R * (int64_t)sizeof(double2);
    if (scratch_bytes < need) return gade_set_error(GADE_ERR_ARG, "gade_pod_project: scratch too small");
    cudaStream_t st = (cudaStream_t)stream;
    if (fp64)
        k_pod_partial64<<<dim3(npulse, nch), 256, 0, st>>>((int)n, R, (const float2 *)U, (const double2 *)x, ldx,
                                                           (double2 *)scratch, npulse);
    else
        k_pod_partial<<<dim3(npulse, nch), 256, 0, st>>>((int)n, R, (const float2 *)U, (const double2 *)x, ldx,
                                                         (double2 *)scratch, npulse);
    LCK("gade_pod_project");
    k_pod_sum<<<(npulse * R + 255) / 256, 256, 0, st>>>(nch, npulse, R, (const double2 *)scratch, (double2 *)coef);
    LCK("gade_pod_project");
    return GADE_OK;
}

extern "C" int gade_pod_project(int64_t n, int32_t R, const void *U, const void *x, int64_t ldx, int32_t npulse,
                                void *coef, void *scratch, int64_t scratch_bytes, void *stream)
{
    return pod_project(false, n, R, U, x, ldx, npulse, coef, scratch, scratch_bytes, stream);
}

extern "C" int gade_pod_project_fp64(int64_t n, int32_t R, const void *U, const void *x, int64_t ldx,
                                     int32_t npulse, void *coef, void *scratch, int64_t scratch_bytes, void *stream)
{
    return pod_project(true, n, R, U, x, ldx, npulse, coef, scratch, scratch_bytes, stream);
}

extern "C" int64_t gade_pod_project_scratch(int64_t n, int32_t R, int32_t npulse)
{
    return ((n + PJ_L - 1) / PJ_L) * (int64_t)npulse * R * (int64_t)sizeof(double2);
}

/* y_p[i] = sum_r U[r][i] c_p[r] for the pulses whose scale is nonzero;
 * complex64 basis and coefficients, complex128 result (stride ldy).  One
 * thread per i walks the basis rows, so U is read once per launch for all
 * the pulses of the block's tile. */
#define EX_PT 8
__global__ void __launch_bounds__(256) k_pod_expand(int n, int R, const float2 *__restrict__ U,
                                                    const float2 *__restrict__ c, const float *__restrict__ scale,
                                                    int npulse, double2 *__restrict__ y, long long ldy)
{
    extern __shared__ float2 cs[];                   /* [EX_PT][R] */
    const int p0 = blockIdx.y * EX_PT;
    const int np = npulse - p0 < EX_PT ? npulse - p0 : EX_PT;
    for (int e = threadIdx.x; e < np * R; e += blockDim.x) {
        const int pp = e / R, r = e % R;
        const float s = scale ? scale[p0 + pp] : 1.f;
        const float2 v = c[(size_t)(p0 + pp) * R + r];
        cs[pp * R + r] = make_float2(s * v.x, s * v.y);
    }
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float ar[EX_PT], ai[EX_PT];
#pragma unroll
        for (int pp = 0; pp < EX_PT; pp++) { ar[pp] = 0.f; ai[pp] = 0.f; }
        for (int r = 0; r < R; r++) {
            const float2 u = U[(size_t)r * n + i];
#pragma unroll
            for (int pp = 0; pp < EX_PT; pp++) {
                if (pp < np) {
                    const float2 cv = cs[pp * R + r];
                    ar[pp] = fmaf(u.x, cv.x, fmaf(-u.y, cv.y, ar[pp]));
                    ai[pp] = fmaf(u.x, cv.y, fmaf(u.y, cv.x, ai[pp]));
                }
            }
        }
#pragma unroll
        for (int pp = 0; pp < EX_PT; pp++)
            if (pp < np) y[(size_t)(p0 + pp) * ldy + i] = make_double2(ar[pp], ai[pp]);
    }
}

extern "C" int gade_pod_expand(int64_t n, int32_t R, const void *U, const void *c, const float *scale,
                               int32_t npulse, void *y, int64_t ldy, void *stream)
{
    if (n <= 0 || n > (1ll << 31) - 1 || R <= 0 || R > 1024 || npulse <= 0 || !U || !c || !y)
        return gade_set_error(GADE_ERR_ARG, "gade_pod_expand: bad argument");
    int gx = (int)((n + 255) / 256);
    if (gx > 1216) gx = 1216;
    const size_t smem = sizeof(float2) * EX_PT * (size_t)R;
    k_pod_expand<<<dim3(gx, (npulse + EX_PT - 1) / EX_PT), 256, smem, (cudaStream_t)stream>>>(
        (int)n, R, (const float2 *)U, (const float2 *)c, scale, npulse, (double2 *)y, ldy);
    LCK("gade_pod_expand");
    return GADE_OK;
}

/* ------------------------------------------------------------------ */
/* network input / output                                              */
/* ------------------------------------------------------------------ */
/* Input row of pulse p: the projections of the last K states (newest
 * first; hist is a ring [K][npulse][R] complex128 whose newest slot is
 * `head`) as (re, im) pairs, then the 12 reals of f(t), all normalised
 * ((v - mu) / sd) and rounded to BF16: row length K*2R + 12. */
__global__ void k_features(int npulse, int R, int K, int head, const double2 *__restrict__ hist,
                           const double *__restrict__ ft, const float *__restrict__ mu, const float *__restrict__ sd,
                           bf16 *__restrict__ out, float *__restrict__ out32)
{
    const int p = blockIdx.x;
    const int D = K * 2 * R + 12;
    for (int e = threadIdx.x; e < D; e += blockDim.x) {
        double v;
        if (e < K * 2 * R) {
            const int j = e / (2 * R), q = e % (2 * R);
            const int slot = (head - j + K) % K;
            const double2 h = hist[((size_t)slot * npulse + p) * R + q / 2];
            v = (q & 1) ? h.y : h.x;
        } else {
            v = ft[(size_t)p * 12 + (e - K * 2 * R)];
        }
        const float z = (float)((v - (double)mu[e]) / (double)sd[e]);
        out[(size_t)p * D + e] = __float2bfloat16(z);
        if (out32) out32[(size_t)p * D + e] = z;
    }
}

extern "C" int gade_learned_features(int32_t npulse, int32_t R, int32_t K, int32_t head, const void *hist,
                                     const double *ft, const float *mu, const float *sd, void *out16, float *out32,
                                     void *stream)
{
    if (npulse <= 0 || R <= 0 || K <= 0 || head < 0 || head >= K || !hist || !ft || !mu || !sd || !out16)
        return gade_set_error(GADE_ERR_ARG, "gade_learned_features: bad argument");
    k_features<<<npulse, 256, 0, (cudaStream_t)stream>>>(npulse, R, K, head, (const double2 *)hist, ft, mu, sd,
                                                         (bf16 *)out16, out32);
    LCK("gade_learned_features");
    return GADE_OK;
}

/* Network output of pulse p (2R normalised reals) -> complex64 POD
 * coefficients c = out * sd + mu.  The correction is kept (scale 1) only
 * while |c| <= limit * |p_0 - p_1| (the projection of the last state
 * change): a prediction larger than the step itself is implausible and the
 * pulse falls back to plain extrapolation (scale 0).  One block per pulse. */
__global__ void k_outputs(int npulse, int R, int K, int head, const float *__restrict__ out,
                          const float *__restrict__ mu, const float *__restrict__ sd, const double2 *__restrict__ hist,
                          float limit, float2 *__restrict__ c, float *__restrict__ scale)
{
    const int p = blockIdx.x;
    __shared__ double sh[2][256];
    double cn = 0, dn = 0;
    const int s0 = head, s1 = (head - 1 + K) % K;
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
        const float re = out[(size_t)p * 2 * R + 2 * r] * sd[2 * r] + mu[2 * r];
        const float im = out[(size_t)p * 2 * R + 2 * r + 1] * sd[2 * r + 1] + mu[2 * r + 1];
        c[(size_t)p * R + r] = make_float2(re, im);
        cn += (double)re * re + (double)im * im;
        const double2 a = hist[((size_t)s0 * npulse + p) * R + r], b = hist[((size_t)s1 * npulse + p) * R + r];
        dn += (a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y);
    }
    sh[0][threadIdx.x] = cn;
    sh[1][threadIdx.x] = dn;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) { sh[0][threadIdx.x] += sh[0][threadIdx.x + w]; sh[1][threadIdx.x] += sh[1][threadIdx.x + w]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const bool ok = isfinite(sh[0][0]) && sh[0][0] <= (double)limit * limit * sh[1][0];
        scale[p] = ok ? 1.f : 0.f;
    }
}

extern "C" int gade_learned_outputs(int32_t npulse, int32_t R, int32_t K, int32_t head, const float *out,
                                    const float *mu, const float *sd, const void *hist, float limit, void *c,
                                    float *scale, void *stream)
{
    if (npulse <= 0 || R <= 0 || K < 2 || head < 0 || head >= K || !out || !mu || !sd || !hist || !c || !scale)
        return gade_set_error(GADE_ERR_ARG, "gade_learned_outputs: bad argument");
    k_outputs<<<npulse, 256, 0, (cudaStream_t)stream>>>(npulse, R, K, head, out, mu, sd, (const double2 *)hist, limit,
                                                        (float2 *)c, scale);
    LCK("gade_learned_outputs");
    return GADE_OK;
}

/* ------------------------------------------------------------------ */
/* eigenstate projection (populations)                                 */
/* ------------------------------------------------------------------ */
/* grid (block row, pulse), 256 threads: the block's slice of x is staged in
 * shared memory; thread t owns eigenvectors j = t, t+256, ... (consecutive
 * threads read consecutive W entries); class sums reduce in fixed order. */
__global__ void __launch_bounds__(256) k_eigproj(int nblk, int B, const int *__restrict__ kidx,
                                                 const double *__restrict__ W, const double *__restrict__ ev,
                                                 double e_lo, const double2 *__restrict__ x, long long ldx,
                                                 double2 *__restrict__ coef, double *__restrict__ classes)
{
    extern __shared__ double2 xs[];                  /* [B] */
    __shared__ double red[4][256];
    const int r = blockIdx.x, p = blockIdx.y, tid = threadIdx.x;
    const int k = kidx[r];
    const double2 *xr = x + (size_t)p * ldx + (size_t)r * B;
    for (int i = tid; i < B; i += 256) xs[i] = xr[i];
    __syncthreads();
    const double *Wk = W + (size_t)k * B * B;
    const double *E = ev + (size_t)k * B;
    double acc[4] = {0, 0, 0, 0};
    for (int j = tid; j < B; j += 256) {
        double cr = 0, ci = 0;
        for (int i = 0; i < B; i++) {
            const double w = Wk[(size_t)i * B + j];
            cr = fma(w, xs[i].x, cr);
            ci = fma(-w, xs[i].y, ci);          /* conj(x) */
        }
        if (coef) coef[((size_t)p * nblk + r) * B + j] = make_double2(cr, ci);
        const double pj = cr * cr + ci * ci;
        const double e = E[j];
        acc[e < e_lo ? 0 : (e < 0.0 ? 1 : 2)] += pj;
        acc[3] += pj;
    }
    for (int c = 0; c < 4; c++) red[c][tid] = acc[c];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (tid < w)
            for (int c = 0; c < 4; c++) red[c][tid] += red[c][tid + w];
        __syncthreads();
    }
    if (tid < 4) classes[((size_t)p * nblk + r) * 4 + tid] = red[tid][0];
}

extern "C" int gade_eigproj(int32_t npulse, int32_t nblk, int32_t B, const int32_t *block_kidx, const double *W,
                            const double *evals, double e_lo, const void *x, int64_t ldx, void *coef,
                            double *classes, void *stream)
{
    if (npulse <= 0 || nblk <= 0 || B <= 0 || B > 2048 || npulse > 65535 || !block_kidx || !W || !evals || !x ||
        !classes)
        return gade_set_error(GADE_ERR_ARG, "gade_eigproj: bad argument");
    k_eigproj<<<dim3(nblk, npulse), 256, sizeof(double2) * (size_t)B, (cudaStream_t)stream>>>(
        nblk, B, block_kidx, W, evals, e_lo, (const double2 *)x, ldx, (double2 *)coef, classes);
    LCK("gade_eigproj");
    return GADE_OK;
}

/* ------------------------------------------------------------------ */
/* the learned guess of a batch, one step per call                      */
/* ------------------------------------------------------------------ */
extern "C" int gade_learned_guess_step(const gade_learned_guess_plan *P, int32_t head, const double *ft, void *stream)
{
    if (!P || head < 0 || head >= P->K || P->npulse < 1 || P->R < 1 || P->din != P->K * 2 * P->R + 12 ||
        P->dout != 2 * P->R)
        return gade_set_error(GADE_ERR_ARG, "gade_learned_guess_step: bad plan");
    const int np = P->npulse, R = P->R;
    void *slot = (char *)P->hist + (size_t)head * np * R * 16;      /* complex128 [npulse][R] */
    int rc = gade_pod_project(P->n, R, P->U, P->x, P->ldx, np, slot, P->scratch, P->scratch_bytes, stream);
    if (rc || !ft) return rc;
    if ((rc = gade_learned_features(np, R, P->K, head, P->hist, ft, P->mu_in, P->sd_in, P->x16, nullptr, stream)))
        return rc;
    /* the network: din -> dh (ReLU) -> dh (ReLU) -> dout, BF16 operands, FP32 accumulation */
    if ((rc = gade_gemm_bf16(np, P->dh, P->din, P->x16, P->din, 1, P->W16[0], P->dh, 1, P->bias[0], nullptr, 0, 1,
                             P->H1, P->dh, P->H1_16, P->dh, stream)))
        return rc;
    if ((rc = gade_gemm_bf16(np, P->dh, P->dh, P->H1_16, P->dh, 1, P->W16[1], P->dh, 1, P->bias[1], nullptr, 0, 1,
                             P->H2, P->dh, P->H2_16, P->dh, stream)))
        return rc;
    if ((rc = gade_gemm_bf16(np, P->dout, P->dh, P->H2_16, P->dh, 1, P->W16[2], P->dout, 1, P->bias[2], nullptr, 0,
                             0, P->out, P->dout, nullptr, 0, stream)))
        return rc;
    if ((rc = gade_learned_outputs(np, R, P->K, head, P->out, P->mu_out, P->sd_out, P->hist, P->limit, P->c,
                                   P->scale, stream)))
        return rc;
    return gade_pod_expand(P->n, R, P->U, P->c, P->scale, np, P->corr, P->ldcorr, stream);
}
