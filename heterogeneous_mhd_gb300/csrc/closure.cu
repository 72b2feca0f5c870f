// The learned closure on the GPU: a periodic 3-D convolution net on the
// coarse state, trained on the GPU by these kernels.
//
// * Convolutions are implicit GEMMs on the BF16 tensor cores with FP32
//   accumulation (mma.sync m16n8k16): M = voxels of a 8x8x4 tile, N = output
//   channels, K = taps x input channels.  A CTA stages the tile and its
//   one-voxel periodic halo (rows of channels, padded so that ldmatrix reads
//   are conflict-free) and the whole weight matrix in shared memory; the
//   ldmatrix row addresses do the im2col gather.  The same kernel runs the
//   forward layers (epilogue: bias + GELU, or bias to FP32 for the head) and
//   the data gradient (flipped, transposed weights; epilogue: times GELU' of
//   the previous layer's saved pre-activation).
// * The weight gradient is a second implicit GEMM, dW = dZ^T im2col(A), with
//   the voxels as the reduction axis; CTAs write deterministic partials that
//   one more kernel sums.
// * Loss (fluid residual + the face residual of the EMF's curl), input
//   features, box filter, correction step and AdamW are plain kernels.
//
// The reference has no closure; the state layout and staggering are those of
// C/mhd.c:26-41 (u(5,...), face-centred b(3,...), component index fastest).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

#include "../../include/mhd_closure.h"
#include "mhd_ptx.cuh"

namespace {

using bf16 = __nv_bfloat16;

// ------------------------------------------------------------ PTX helpers

__device__ __forceinline__ void cp_async16(void* dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(mhd::smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_all;" ::: "memory");
}

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void* p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(mhd::smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x2(uint32_t (&r)[2], const void* p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];"
                 : "=r"(r[0]), "=r"(r[1])
                 : "r"(mhd::smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const void* p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(mhd::smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z)
{
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

__device__ __forceinline__ float mhd_warp_sum(float x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}
__device__ __forceinline__ double mhd_warp_sum_d(double x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// ------------------------------------------------------------ tiles

constexpr int TX = 8, TY = 8, TZ = 4;  // voxels of a tile (x fastest)
constexpr int TV = TX * TY * TZ;       // 256

template <int KS>
struct Halo {
    static constexpr int H = KS - 1;
    static constexpr int X = TX + H, Y = TY + H, Z = TZ + H;
    static constexpr int ROWS = X * Y * Z;
};

// bytes of one smem row of C bf16 channels: padded by 16 B so that eight
// consecutive rows fall into distinct bank quads (ldmatrix without conflicts)
__host__ __device__ constexpr int row_bytes(int c) { return c * 2 + 16; }

struct TileIdx {
    int box, z0, y0, x0;
};
__device__ __forceinline__ TileIdx tile_of(long long t, int n)
{
    const int tx = n / TX, ty = n / TY, tz = n / TZ;
    TileIdx r;
    r.x0 = (int)(t % tx) * TX;
    t /= tx;
    r.y0 = (int)(t % ty) * TY;
    t /= ty;
    r.z0 = (int)(t % tz) * TZ;
    r.box = (int)(t / tz);
    return r;
}
__device__ __forceinline__ int wrap(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// Stage the tile's rows (with halo for KS = 3) of a [box][n^3][C] bf16 tensor.
template <int C, int KS>
__device__ __forceinline__ void load_rows(unsigned char* dst, const bf16* src, const TileIdx& t, int n)
{
    using HL = Halo<KS>;
    constexpr int CH = C * 2 / 16;  // 16-byte chunks per row
    const int h = KS / 2;
    const size_t box0 = (size_t)t.box * n * n * n;
    for (int e = threadIdx.x; e < HL::ROWS * CH; e += blockDim.x) {
        const int row = e / CH, ch = e - row * CH;
        const int hx = row % HL::X, r2 = row / HL::X, hy = r2 % HL::Y, hz = r2 / HL::Y;
        const int x = wrap(t.x0 + hx - h, n), y = wrap(t.y0 + hy - h, n), z = wrap(t.z0 + hz - h, n);
        const bf16* s = src + (box0 + ((size_t)z * n + y) * n + x) * C + ch * 8;
        cp_async16(dst + (size_t)row * row_bytes(C) + ch * 16, s);
    }
}

enum Epi { EPI_GELU = 0, EPI_LINEAR_F32 = 1, EPI_DGRAD = 2 };

// y(v, co) = sum_{tap, ci} x(v + off(tap), ci) W(co, tap, ci); W is [COUT][KS^3][CIN] bf16.
template <int CIN, int COUT, int KS, int EPI>
__global__ void __launch_bounds__(128) k_conv(const bf16* __restrict__ x, const bf16* __restrict__ w,
                                              const float* __restrict__ bias, void* __restrict__ y,
                                              bf16* __restrict__ zsave, const bf16* __restrict__ zprev, int n,
                                              long long ntiles)
{
    using HL = Halo<KS>;
    constexpr int TAPS = KS * KS * KS;
    constexpr int RS = row_bytes(CIN);
    constexpr int WRS = TAPS * CIN * 2 + 16;
    constexpr int NT = COUT / 8;  // n-tiles
    constexpr int MT = 4;         // m-tiles (of 16 voxels) per warp
    extern __shared__ __align__(16) unsigned char sm[];
    unsigned char* sx = sm;                                // [ROWS][RS]
    unsigned char* sw = sm + (size_t)HL::ROWS * RS;        // [COUT][WRS]

    // weights once per CTA
    {
        constexpr int CHW = TAPS * CIN * 2 / 16;
        for (int e = threadIdx.x; e < COUT * CHW; e += blockDim.x) {
            const int r = e / CHW, c = e - r * CHW;
            cp_async16(sw + (size_t)r * WRS + c * 16, reinterpret_cast<const unsigned char*>(w) +
                                                          ((size_t)r * TAPS * CIN * 2 + c * 16));
        }
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tz = warp;  // each warp: one z-slice of 8x8 voxels
    // ldmatrix lane roles
    const int ar = (lane & 7) + ((lane >> 3) & 1) * 8, ak = (lane >> 4) * 8;      // A: row, k offset
    const int bn = (lane & 7) + ((lane >> 4) << 3), bk = ((lane >> 3) & 1) * 8;   // B (x4): n, k offset
    const int bn2 = lane & 7, bk2 = ((lane >> 3) & 1) * 8;                          // B (x2)

    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const TileIdx t = tile_of(tile, n);
        __syncthreads();  // previous tile's readers are done with sx
        load_rows<CIN, KS>(sx, x, t, n);
        cp_async_wait_all();
        __syncthreads();

        float acc[MT][NT][4];
#pragma unroll
        for (int i = 0; i < MT; i++)
#pragma unroll
            for (int j = 0; j < NT; j++)
#pragma unroll
                for (int q = 0; q < 4; q++)
                    acc[i][j][q] = 0.f;

#pragma unroll 1
        for (int tap = 0; tap < TAPS; tap++) {
            const int dk = tap / (KS * KS), dj = (tap / KS) % KS, di = tap % KS;
#pragma unroll
            for (int kc = 0; kc < CIN / 16; kc++) {
                uint32_t bfr[NT][2];
                if constexpr (NT == 1) {
                    uint32_t r[2];
                    ldsm_x2(r, sw + (size_t)bn2 * WRS + ((tap * CIN + kc * 16 + bk2) * 2));
                    bfr[0][0] = r[0];
                    bfr[0][1] = r[1];
                } else {
#pragma unroll
                    for (int j = 0; j < NT; j += 2) {
                        uint32_t r[4];
                        ldsm_x4(r, sw + (size_t)(j * 8 + bn) * WRS + ((tap * CIN + kc * 16 + bk) * 2));
                        bfr[j][0] = r[0];
                        bfr[j][1] = r[1];
                        bfr[j + 1][0] = r[2];
                        bfr[j + 1][1] = r[3];
                    }
                }
#pragma unroll
                for (int i = 0; i < MT; i++) {
                    const int ty = 2 * i + (ar >> 3), tx = ar & 7;
                    const int row = ((tz + dk) * HL::Y + (ty + dj)) * HL::X + (tx + di);
                    uint32_t a[4];
                    ldsm_x4(a, sx + (size_t)row * RS + (kc * 16 + ak) * 2);
#pragma unroll
                    for (int j = 0; j < NT; j++)
                        mma_bf16(acc[i][j], a, bfr[j][0], bfr[j][1]);
                }
            }
        }

        // epilogue: rows lane/4 and lane/4 + 8 of each m-tile, channel pair 2*(lane%4)
        const size_t box0 = (size_t)t.box * n * n * n;
#pragma unroll
        for (int i = 0; i < MT; i++)
#pragma unroll
            for (int hr = 0; hr < 2; hr++) {
                const int r = (lane >> 2) + 8 * hr;
                const int ty = 2 * i + (r >> 3), tx = r & 7;
                const size_t v = box0 + ((size_t)(t.z0 + tz) * n + (t.y0 + ty)) * n + (t.x0 + tx);
#pragma unroll
                for (int j = 0; j < NT; j++) {
                    const int co = j * 8 + 2 * (lane & 3);
                    float v0 = acc[i][j][2 * hr], v1 = acc[i][j][2 * hr + 1];
                    if constexpr (EPI == EPI_GELU) {
                        const __nv_bfloat162 z = __floats2bfloat162_rn(v0 + bias[co], v1 + bias[co + 1]);
                        *reinterpret_cast<__nv_bfloat162*>(zsave + v * COUT + co) = z;
                        const float2 zf = __bfloat1622float2(z);
                        *reinterpret_cast<__nv_bfloat162*>(static_cast<bf16*>(y) + v * COUT + co) =
                            __floats2bfloat162_rn(gelu(zf.x), gelu(zf.y));
                    } else if constexpr (EPI == EPI_LINEAR_F32) {
                        *reinterpret_cast<float2*>(static_cast<float*>(y) + v * COUT + co) =
                            make_float2(v0 + bias[co], v1 + bias[co + 1]);
                    } else {
                        const float2 zp =
                            __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(zprev + v * COUT + co));
                        *reinterpret_cast<__nv_bfloat162*>(static_cast<bf16*>(y) + v * COUT + co) =
                            __floats2bfloat162_rn(v0 * gelu_grad(zp.x), v1 * gelu_grad(zp.y));
                    }
                }
            }
    }
}

// ------------------------------------------------------------ tcgen05 path
//
// The same 3^3 convolution on the 5th-generation tensor cores.  A persistent
// CTA (8 warps) takes tiles of 16 (x) x 8 (y) x 2 (z) voxels: two M = 128
// blocks (one per plane, rows m = 8 x + y).  Its halo tile (18 x 10 x 4
// voxels) sits in shared memory chunk-major, [channel chunk of 8][z'][x'][y']
// x 16 B, so for every plane and tap (dk, dj, di) the A operand is one
// K-major no-swizzle descriptor: 8-row core matrices are 8 consecutive y'
// (128 B), the 16 row groups (x) are 160 B apart (SBO) and the two 8-channel
// chunks of a K-step one chunk apart (LBO); plane and tap only move the start
// address, a compile-time offset.  The weights ([K chunk][cout] x 16 B) stay
// resident.  One thread issues the 2 x 27 x CIN/16 MMAs (M = 128, N = COUT,
// K = 16, BF16 in, FP32 accumulate) into one of two TMEM buffers and commits
// them to that buffer's mbarrier; meanwhile all warps run the epilogue of the
// previous tile from the other buffer (tcgen05.ld 32x32b: warp w reads plane
// w / 4, lanes 32 (w % 4)..) and the next tile's halo arrives by cp.async
// into the other shared buffer.  Waits are bounded: on timeout the kernel
// records DEVERR_TIMEOUT, stops and frees its TMEM.

constexpr int TCX = 16, TCY = 8, TCZ = 2;                    // tile
constexpr int HX = TCX + 2, HY = TCY + 2, HZ = TCZ + 2;      // halo tile
constexpr int HV = HX * HY * HZ;                             // 720 voxels
constexpr uint32_t kChunkBytes = HV * 16;                    // one 8-channel chunk of the halo

__device__ __forceinline__ uint64_t umma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

__device__ __forceinline__ void umma_f16(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc, int acc)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                 "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

// (t0, nt: this thread's index among the nt threads that share the copies)
template <int CIN>
__device__ __forceinline__ void tc_load_halo(unsigned char* dst, const bf16* src, int box, int z0, int y0, int x0,
                                             int n, int t0, int nt)
{
    constexpr int CH = CIN / 8;
    const size_t box0 = (size_t)box * n * n * n;
    // consecutive threads: chunks of one voxel, then x (contiguous rows in HBM)
    for (int e = t0; e < HV * CH; e += nt) {
        const int c = e % CH, r = e / CH;
        const int xp = r % HX, r2 = r / HX, yp = r2 % HY, zp = r2 / HY;
        const int gx = wrap(x0 + xp - 1, n), gy = wrap(y0 + yp - 1, n), gz = wrap(z0 + zp - 1, n);
        const bf16* s = src + (box0 + ((size_t)gz * n + gy) * n + gx) * CIN + c * 8;
        cp_async16(dst + c * kChunkBytes + ((zp * HX + xp) * HY + yp) * 16, s);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// all MMAs of one tile: plane P, tap T, K-step KS; offsets are compile-time
template <int CIN, int COUT>
__device__ __forceinline__ void tc_issue_tile(uint32_t tmem, uint64_t a_desc0, uint64_t b_desc0, uint32_t idesc)
{
    constexpr int CH = CIN / 8;
#pragma unroll
    for (int p = 0; p < TCZ; p++)
#pragma unroll
        for (int tap = 0; tap < 27; tap++)
#pragma unroll
            for (int ks = 0; ks < CIN / 16; ks++) {
                const int dk = tap / 9, dj = (tap / 3) % 3, di = tap % 3;
                const uint32_t aoff = (((dk + p) * HX + di) * HY + dj) * 16 + 2 * ks * kChunkBytes;
                const uint32_t boff = (uint32_t)(tap * CH + 2 * ks) * COUT * 16;
                umma_f16(tmem + 32 * p, a_desc0 + (aoff >> 4), b_desc0 + (boff >> 4), idesc, tap | ks);
            }
}

// The epilogue of one voxel: its COUT accumulators (FP32 bits) to bias + GELU
// in BF16 (and the pre-activation for the backward pass), or times GELU' of
// the previous layer's pre-activation (the data gradient).
template <int COUT, int EPI>
__device__ __forceinline__ void tc_epilogue_row(const uint32_t (&r)[32], size_t v, const float* __restrict__ bias,
                                                void* __restrict__ y, bf16* __restrict__ zsave,
                                                const bf16* __restrict__ zprev)
{
    __align__(16) bf16 o1[COUT];
    __align__(16) bf16 o2[COUT];
#pragma unroll
    for (int c = 0; c < COUT; c += 2) {
        const float v0 = __uint_as_float(r[c]), v1 = __uint_as_float(r[c + 1]);
        if constexpr (EPI == EPI_GELU) {
            const __nv_bfloat162 zz = __floats2bfloat162_rn(v0 + bias[c], v1 + bias[c + 1]);
            const float2 zf = __bfloat1622float2(zz);
            *reinterpret_cast<__nv_bfloat162*>(o2 + c) = zz;
            *reinterpret_cast<__nv_bfloat162*>(o1 + c) = __floats2bfloat162_rn(gelu(zf.x), gelu(zf.y));
        } else {
            const float2 zp = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(zprev + v * COUT + c));
            *reinterpret_cast<__nv_bfloat162*>(o1 + c) =
                __floats2bfloat162_rn(v0 * gelu_grad(zp.x), v1 * gelu_grad(zp.y));
        }
    }
    uint4* yo = reinterpret_cast<uint4*>(static_cast<bf16*>(y) + v * COUT);
#pragma unroll
    for (int k = 0; k < COUT / 8; k++)
        yo[k] = reinterpret_cast<const uint4*>(o1)[k];
    if constexpr (EPI == EPI_GELU) {
        uint4* zo = reinterpret_cast<uint4*>(zsave + v * COUT);
#pragma unroll
        for (int k = 0; k < COUT / 8; k++)
            zo[k] = reinterpret_cast<const uint4*>(o2)[k];
    }
}

// The same epilogue with GELU and GELU' read from tables indexed by the BF16
// bits of the pre-activation (gelu_tab: the BF16 bits of gelu, grad_tab: the
// FP32 gelu'), which hold exactly what gelu() and gelu_grad() give on those
// 65536 inputs: the results are the computed epilogue's bit for bit.
template <int COUT, int EPI>
__device__ __forceinline__ void tc_epilogue_row_tab(const uint32_t (&r)[32], size_t v, const float* __restrict__ bias,
                                                    void* __restrict__ y, bf16* __restrict__ zsave,
                                                    const bf16* __restrict__ zprev,
                                                    const unsigned short* __restrict__ gelu_tab,
                                                    const float* __restrict__ grad_tab)
{
    __align__(16) bf16 o1[COUT];
    __align__(16) bf16 o2[COUT];
#pragma unroll
    for (int c = 0; c < COUT; c += 2) {
        const float v0 = __uint_as_float(r[c]), v1 = __uint_as_float(r[c + 1]);
        if constexpr (EPI == EPI_GELU) {
            const __nv_bfloat162 zz = __floats2bfloat162_rn(v0 + bias[c], v1 + bias[c + 1]);
            *reinterpret_cast<__nv_bfloat162*>(o2 + c) = zz;
            const uint32_t bits = *reinterpret_cast<const uint32_t*>(&zz);
            const uint32_t g = (uint32_t)__ldg(gelu_tab + (bits & 0xFFFFu)) |
                               ((uint32_t)__ldg(gelu_tab + (bits >> 16)) << 16);
            *reinterpret_cast<uint32_t*>(o1 + c) = g;
        } else {
            const uint32_t zb = *reinterpret_cast<const uint32_t*>(zprev + v * COUT + c);
            *reinterpret_cast<__nv_bfloat162*>(o1 + c) =
                __floats2bfloat162_rn(v0 * __ldg(grad_tab + (zb & 0xFFFFu)), v1 * __ldg(grad_tab + (zb >> 16)));
        }
    }
    uint4* yo = reinterpret_cast<uint4*>(static_cast<bf16*>(y) + v * COUT);
#pragma unroll
    for (int k = 0; k < COUT / 8; k++)
        yo[k] = reinterpret_cast<const uint4*>(o1)[k];
    if constexpr (EPI == EPI_GELU) {
        uint4* zo = reinterpret_cast<uint4*>(zsave + v * COUT);
#pragma unroll
        for (int k = 0; k < COUT / 8; k++)
            zo[k] = reinterpret_cast<const uint4*>(o2)[k];
    }
}

// gelu and gelu' of every BF16 value (the tables of tc_epilogue_row_tab)
__global__ void k_gelu_tables(unsigned short* __restrict__ gelu_tab, float* __restrict__ grad_tab)
{
    const int code = blockIdx.x * blockDim.x + threadIdx.x;
    if (code >= 65536)
        return;
    const unsigned short b = (unsigned short)code;
    const float z = __bfloat162float(*reinterpret_cast<const bf16*>(&b));
    const bf16 g = __float2bfloat16_rn(gelu(z));
    gelu_tab[code] = *reinterpret_cast<const unsigned short*>(&g);
    grad_tab[code] = gelu_grad(z);
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
                 "%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
                   "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
                   "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(256, 1) k_conv_tc(const bf16* __restrict__ x, const bf16* __restrict__ w,
                                                     const float* __restrict__ bias, void* __restrict__ y,
                                                     bf16* __restrict__ zsave, const bf16* __restrict__ zprev, int n,
                                                     long long ntiles, int* err)
{
    static_assert(COUT == 32, "one tile's accumulators are 2 x 32 TMEM columns");
    constexpr int CH = CIN / 8;
    constexpr int KC = 27 * CH;                  // K chunks of the weights
    constexpr uint32_t ABYTES = CH * kChunkBytes;
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char* sW = sm + 2 * ABYTES;         // [KC][COUT][16 B]
    __shared__ __align__(8) uint64_t mma_bar[2];
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // weights: global [COUT][27][CIN] bf16 -> [K chunk][cout] x 16 B
    for (int e = tid; e < KC * COUT; e += blockDim.x) {
        const int co = e % COUT, kc = e / COUT;
        cp_async16(sW + ((size_t)kc * COUT + co) * 16, w + (size_t)co * 27 * CIN + kc * 8);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    if (tid == 0) {
        for (int b = 0; b < 2; b++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mhd::smem_u32(&mma_bar[b])));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(
                         mhd::smem_u32(&tmem_base)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(COUT >> 3) << 17) | (8u << 24);
    const uint64_t a_desc[2] = {umma_desc(mhd::smem_u32(sm), kChunkBytes, HY * 16),
                                umma_desc(mhd::smem_u32(sm + ABYTES), kChunkBytes, HY * 16)};
    const uint64_t b_desc = umma_desc(mhd::smem_u32(sW), COUT * 16, 128);

    const int tx = n / TCX, ty = n / TCY, tz = n / TCZ;
    auto coords = [&](long long t, int& box, int& z0, int& y0, int& x0) {
        x0 = (int)(t % tx) * TCX;
        t /= tx;
        y0 = (int)(t % ty) * TCY;
        t /= ty;
        z0 = (int)(t % tz) * TCZ;
        box = (int)(t / tz);
    };
    if ((long long)blockIdx.x < ntiles) {
        int b_, z_, y_, x_;
        coords(blockIdx.x, b_, z_, y_, x_);
        tc_load_halo<CIN>(sm, x, b_, z_, y_, x_, n, tid, blockDim.x);
    }
    int pbox = 0, pz = 0, py = 0, px = 0;  // the previous tile (its epilogue runs this iteration)
    for (long long it = 0;; it++) {
        const long long tile = blockIdx.x + it * gridDim.x;
        const bool cur = tile < ntiles;
        const int ab = (int)(it & 1);
        // (1) the previous tile's MMAs: its A buffer is refilled and its TMEM read below
        if (it > 0) {
            const int pb = (int)((it - 1) & 1);
            const bool ok = mhd::mbar_wait_bounded(&mma_bar[pb], (uint32_t)(((it - 1) >> 1) & 1), err);
            if (__syncthreads_or(!ok))
                break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        }
        // (2) prefetch the next tile into the other A buffer; (3) wait for this tile's halo
        int box = 0, z0 = 0, y0 = 0, x0 = 0;
        if (cur) {
            coords(tile, box, z0, y0, x0);
            const long long next = tile + gridDim.x;
            if (next < ntiles) {
                int b_, z_, y_, x_;
                coords(next, b_, z_, y_, x_);
                tc_load_halo<CIN>(sm + (ab ^ 1) * ABYTES, x, b_, z_, y_, x_, n, tid, blockDim.x);
                asm volatile("cp.async.wait_group 1;" ::: "memory");
            } else {
                asm volatile("cp.async.wait_group 0;" ::: "memory");
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // cp.async writes -> tensor core
        }
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // (4) this tile's MMAs into TMEM columns 64 ab .. 64 ab + 63
        if (cur && tid == 0) {
            tc_issue_tile<CIN, COUT>(tmem + 64 * ab, a_desc[ab], b_desc, idesc);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             mhd::smem_u32(&mma_bar[ab]))
                         : "memory");
        }
        // (5) epilogue of the previous tile
        if (it > 0) {
            const int pb = (int)((it - 1) & 1), pl = warp >> 2, q = warp & 3;
            uint32_t r[32];
            const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + 64 * pb + 32 * pl;
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
                         "%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                           "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                           "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
                           "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
                           "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                         : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            const int m = q * 32 + lane, vx = m >> 3, vy = m & 7;
            const size_t v = (((size_t)pbox * n + pz + pl) * n + (py + vy)) * n + (px + vx);
            tc_epilogue_row<COUT, EPI>(r, v, bias, y, zsave, zprev);
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (!cur)
            break;
        pbox = box, pz = z0, py = y0, px = x0;
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem));
}

// The same convolution as a warp-specialised pipeline, so that the tensor
// core does not wait for the epilogue or for the halo loads.  Nine warps:
//   * warps 0-3 load halo tiles by cp.async into a ring of NA shared buffers
//     (a stage is announced on a_full once its copies have landed, with one
//     stage of lag so that two tiles' loads are in flight);
//   * warp 4 (one elected lane) issues a tile's 2 x 27 x CIN/16 MMAs into
//     one of NT TMEM stages of 64 columns as soon as its halo is in and the
//     stage is free, then commits them to a_empty (the halo buffer is free)
//     and t_full (the accumulators are ready);
//   * warps 5-8 run the epilogue of a TMEM stage (warp w reads lanes
//     32 (w % 4).. of both planes) and free the stage on t_empty as soon as
//     its accumulators are in registers.
// The weights stay resident.  Every wait is bounded: on timeout the role
// records DEVERR_TIMEOUT and leaves its loop, the others then time out in
// turn, and the CTA frees its TMEM after its last MMAs have completed.
constexpr int kTc2Load = 4;                  // loader warps
constexpr int kTc2Warps = kTc2Load + 1 + 4;  // + the MMA warp + four epilogue warps
constexpr int kTc2NT = 4;                    // TMEM stages (4 x 64 = 256 columns)

template <int CIN>
__host__ __device__ constexpr int tc2_stages() { return CIN >= 32 ? 3 : 4; }  // halo buffers: 3 x 45 KB + 54 KB of weights

template <int CIN, int COUT>
__host__ __device__ constexpr size_t tc2_smem_bytes()
{
    return (size_t)tc2_stages<CIN>() * (CIN / 8) * kChunkBytes + (size_t)27 * (CIN / 8) * COUT * 16 + 1024;
}

__device__ __forceinline__ void mbar_arrive1(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mhd::smem_u32(bar)) : "memory");
}

template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(kTc2Warps * 32, 1)
    k_conv_tc2(const bf16* __restrict__ x, const bf16* __restrict__ w, const float* __restrict__ bias,
               void* __restrict__ y, bf16* __restrict__ zsave, const bf16* __restrict__ zprev, int n, long long ntiles,
               int* err, const unsigned short* __restrict__ gelu_tab, const float* __restrict__ grad_tab)
{
    static_assert(COUT == 32, "one tile's accumulators are 2 x 32 TMEM columns");
    constexpr int CH = CIN / 8, NA = tc2_stages<CIN>(), NT = kTc2NT;
    constexpr int KC = 27 * CH;                  // K chunks of the weights
    constexpr uint32_t ABYTES = CH * kChunkBytes;
    constexpr int MMA_WARP = kTc2Load, LOADERS = kTc2Load * 32;
    extern __shared__ __align__(16) unsigned char tc2_raw[];
    // 1024-byte aligned start, as an offset from the shared array
    unsigned char* const sm =
        tc2_raw + ((1024u - (static_cast<uint32_t>(__cvta_generic_to_shared(tc2_raw)) & 1023u)) & 1023u);
    unsigned char* const sW = sm + NA * ABYTES;  // [KC][COUT][16 B]
    __shared__ __align__(8) uint64_t a_full[NA], a_empty[NA], t_full[NT], t_empty[NT];
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    for (int e = tid; e < KC * COUT; e += blockDim.x) {
        const int co = e % COUT, kc = e / COUT;
        cp_async16(sW + ((size_t)kc * COUT + co) * 16, w + (size_t)co * 27 * CIN + kc * 8);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // cp.async writes -> tensor core
    if (tid == 0) {
        for (int i = 0; i < NA; i++) {
            mhd::mbar_init(&a_full[i], LOADERS);
            mhd::mbar_init(&a_empty[i], 1);
        }
        for (int i = 0; i < NT; i++) {
            mhd::mbar_init(&t_full[i], 1);
            mhd::mbar_init(&t_empty[i], 4);
        }
    }
    if (warp == MMA_WARP) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(
                         mhd::smem_u32(&tmem_base)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;
    const int tx = n / TCX, ty = n / TCY, tz = n / TCZ;
    auto coords = [&](long long t, int& box, int& z0, int& y0, int& x0) {
        x0 = (int)(t % tx) * TCX;
        t /= tx;
        y0 = (int)(t % ty) * TCY;
        t /= ty;
        z0 = (int)(t % tz) * TCZ;
        box = (int)(t / tz);
    };
    const long long mine = (ntiles - (long long)blockIdx.x + gridDim.x - 1) / gridDim.x;  // tiles of this CTA
    long long issued = 0;  // tiles whose MMAs the MMA warp committed

    if (warp < kTc2Load) {
        // ---- loaders: halo tiles into the ring, one stage of lag on the announcement
        for (long long i = 0; i < mine; i++) {
            const int sa = (int)(i % NA);
            if (i >= NA && !mhd::mbar_wait_bounded(&a_empty[sa], (uint32_t)(((i / NA) - 1) & 1), err))
                break;
            int b_, z_, y_, x_;
            coords((long long)blockIdx.x + i * gridDim.x, b_, z_, y_, x_);
            tc_load_halo<CIN>(sm + sa * ABYTES, x, b_, z_, y_, x_, n, tid, LOADERS);  // one commit group
            if (i >= 1) {  // the previous tile's copies have landed: announce it
                asm volatile("cp.async.wait_group 1;" ::: "memory");
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive1(&a_full[(int)((i - 1) % NA)]);
            }
        }
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (mine > 0)
            mbar_arrive1(&a_full[(int)((mine - 1) % NA)]);
    } else if (warp == MMA_WARP) {
        // ---- MMA issuer
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(COUT >> 3) << 17) | (8u << 24);
        const uint64_t b_desc = umma_desc(mhd::smem_u32(sW), COUT * 16, 128);
        for (long long i = 0; i < mine; i++) {
            const int sa = (int)(i % NA), st = (int)(i % NT);
            if (!mhd::mbar_wait_bounded(&a_full[sa], (uint32_t)((i / NA) & 1), err))
                break;
            if (i >= NT && !mhd::mbar_wait_bounded(&t_empty[st], (uint32_t)(((i / NT) - 1) & 1), err))
                break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (lane == 0) {
                tc_issue_tile<CIN, COUT>(tmem + 64 * st, umma_desc(mhd::smem_u32(sm + sa * ABYTES), kChunkBytes, HY * 16),
                                         b_desc, idesc);
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 mhd::smem_u32(&a_empty[sa]))
                             : "memory");
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 mhd::smem_u32(&t_full[st]))
                             : "memory");
            }
            __syncwarp();
            issued = i + 1;
        }
        // the last committed MMAs have completed before TMEM is freed
        if (issued > 0)
            mhd::mbar_wait_bounded(&t_full[(int)((issued - 1) % NT)], (uint32_t)(((issued - 1) / NT) & 1), err);
    } else {
        // ---- epilogue: lanes 32 (warp % 4).. of both planes
        const int q = warp & 3;
        for (long long i = 0; i < mine; i++) {
            const int st = (int)(i % NT);
            if (!mhd::mbar_wait_bounded(&t_full[st], (uint32_t)((i / NT) & 1), err))
                break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            uint32_t r0[32], r1[32];
            tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + 64 * st, r0);
            tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + 64 * st + 32, r1);
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0)
                mbar_arrive1(&t_empty[st]);
            int box, z0, y0, x0;
            coords((long long)blockIdx.x + i * gridDim.x, box, z0, y0, x0);
            const int m = q * 32 + lane, vx = m >> 3, vy = m & 7;
            const size_t v = (((size_t)box * n + z0) * n + (y0 + vy)) * n + (x0 + vx);
            tc_epilogue_row_tab<COUT, EPI>(r0, v, bias, y, zsave, zprev, gelu_tab, grad_tab);
            tc_epilogue_row_tab<COUT, EPI>(r1, v + (size_t)n * n, bias, y, zsave, zprev, gelu_tab, grad_tab);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == MMA_WARP)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
}

// dW(co, tap, ci) = sum_v dz(v, co) a(v + off(tap), ci).  Warp w owns the taps
// t == w mod WT and the k-steps (16 voxels) s == w / WT mod WK.  Each warp
// writes its FP32 partial sums to part[cta][w / WT][tap][co][ci].
template <int CIN, int COUTP, int KS>
struct WgradShape {
    static constexpr int TAPS = KS * KS * KS;
    static constexpr int WT = (TAPS >= 9) ? 9 : TAPS;     // warps along taps
    static constexpr int WK = (TAPS >= 9) ? 1 : 8;        // warps along voxels
    static constexpr int TPW = (TAPS + WT - 1) / WT;      // taps per warp
    static constexpr int THREADS = 32 * WT * WK;
};

template <int CIN, int COUTP, int KS>
__global__ void __launch_bounds__(WgradShape<CIN, COUTP, KS>::THREADS)
    k_wgrad(const bf16* __restrict__ a, const bf16* __restrict__ dz, float* __restrict__ part, int n,
            long long ntiles)
{
    using S = WgradShape<CIN, COUTP, KS>;
    using HL = Halo<KS>;
    constexpr int RS = row_bytes(CIN), RZ = row_bytes(COUTP);
    constexpr int MTL = COUTP / 16, NTL = CIN / 8;
    extern __shared__ __align__(16) unsigned char sm[];
    unsigned char* sa = sm;                               // [ROWS][RS]
    unsigned char* sz = sm + (size_t)HL::ROWS * RS;       // [TV][RZ]

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wt = warp % S::WT, wk = warp / S::WT;
    // ldmatrix.trans lane roles: A = dz^T (rows = voxels, cols = co), B = a (rows = voxels, cols = ci)
    const int ak = (lane & 7) + ((lane >> 4) & 1) * 8, am = ((lane >> 3) & 1) * 8;
    const int bk = (lane & 7) + ((lane >> 3) & 1) * 8, bnn = (lane >> 4) * 8;

    float acc[S::TPW][MTL][NTL][4];
#pragma unroll
    for (int p = 0; p < S::TPW; p++)
#pragma unroll
        for (int i = 0; i < MTL; i++)
#pragma unroll
            for (int j = 0; j < NTL; j++)
#pragma unroll
                for (int q = 0; q < 4; q++)
                    acc[p][i][j][q] = 0.f;

    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const TileIdx t = tile_of(tile, n);
        __syncthreads();
        load_rows<CIN, KS>(sa, a, t, n);
        {
            constexpr int CH = COUTP * 2 / 16;
            const size_t box0 = (size_t)t.box * n * n * n;
            for (int e = threadIdx.x; e < TV * CH; e += blockDim.x) {
                const int row = e / CH, ch = e - row * CH;
                const int tx = row % TX, ty = (row / TX) % TY, tz = row / (TX * TY);
                const bf16* s = dz + (box0 + ((size_t)(t.z0 + tz) * n + (t.y0 + ty)) * n + (t.x0 + tx)) * COUTP + ch * 8;
                cp_async16(sz + (size_t)row * RZ + ch * 16, s);
            }
        }
        cp_async_wait_all();
        __syncthreads();

#pragma unroll 1
        for (int s = wk; s < TV / 16; s += S::WK) {
            // A fragments: voxels 16s..16s+15 (tz = s/4, ty = 2(s%4) + r/8, tx = r%8)
            uint32_t af[MTL][4];
#pragma unroll
            for (int i = 0; i < MTL; i++)
                ldsm_x4_t(af[i], sz + (size_t)(16 * s + ak) * RZ + (i * 16 + am) * 2);
            const int r = bk;  // voxel row of this lane's B address
            const int tz = s >> 2, ty = 2 * (s & 3) + (r >> 3), tx = r & 7;
#pragma unroll
            for (int p = 0; p < S::TPW; p++) {
                const int tap = wt + p * S::WT;
                if (tap >= S::TAPS)
                    break;
                const int dk = tap / (KS * KS), dj = (tap / KS) % KS, di = tap % KS;
                const int row = ((tz + dk) * HL::Y + (ty + dj)) * HL::X + (tx + di);
#pragma unroll
                for (int j = 0; j < NTL; j += 2) {
                    uint32_t b[4];
                    ldsm_x4_t(b, sa + (size_t)row * RS + (j * 8 + bnn) * 2);
#pragma unroll
                    for (int i = 0; i < MTL; i++) {
                        mma_bf16(acc[p][i][j], af[i], b[0], b[1]);
                        mma_bf16(acc[p][i][j + 1], af[i], b[2], b[3]);
                    }
                }
            }
        }
    }
    // partials: part[cta][wk][tap][co][ci]
    float* base = part + ((size_t)blockIdx.x * S::WK + wk) * S::TAPS * COUTP * CIN;
#pragma unroll
    for (int p = 0; p < S::TPW; p++) {
        const int tap = wt + p * S::WT;
        if (tap >= S::TAPS)
            break;
#pragma unroll
        for (int i = 0; i < MTL; i++)
#pragma unroll
            for (int j = 0; j < NTL; j++)
#pragma unroll
                for (int hr = 0; hr < 2; hr++) {
                    const int co = i * 16 + (lane >> 2) + 8 * hr, ci = j * 8 + 2 * (lane & 3);
                    float* d = base + ((size_t)tap * COUTP + co) * CIN + ci;
                    d[0] = acc[p][i][j][2 * hr];
                    d[1] = acc[p][i][j][2 * hr + 1];
                }
    }
}

// Partial sums of reductions: a CTA of kSumWarps warps takes 32 consecutive
// output elements; warp w sums the partials p = w, w + kSumWarps, ... of its
// lane's element and the warps' sums are added in warp order (a fixed order:
// deterministic).
constexpr int kSumWarps = 8;

// out[e] = sum_p part[p * stride + e], e < len; launched on (len + 31) / 32 CTAs of kSumWarps warps
__global__ void __launch_bounds__(kSumWarps * 32) k_sum_parts(const float* __restrict__ part, int nparts,
                                                             size_t stride, size_t len, float* __restrict__ out)
{
    __shared__ float red[kSumWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const size_t e = (size_t)blockIdx.x * 32 + lane;
    float s = 0.f;
    if (e < len)
        for (int p = w; p < nparts; p += kSumWarps)
            s += part[(size_t)p * stride + e];
    red[w][lane] = s;
    __syncthreads();
    if (w == 0 && e < len) {
        float t = 0.f;
#pragma unroll
        for (int k = 0; k < kSumWarps; k++)
            t += red[k][lane];
        out[e] = t;
    }
}

// weight-gradient partials part[p][tap][cop][cip] summed into the master
// layout dw[co][tap][ci] for co < cor, ci < cir, in the order of k_sum_parts
// (a coalesced 128-byte row per partial and warp)
constexpr int kWsumWarps = kSumWarps;
__global__ void __launch_bounds__(kWsumWarps * 32) k_wsum(const float* __restrict__ part, int nparts, int taps,
                                                         int cop, int cip, int cor, int cir, float* __restrict__ dw)
{
    __shared__ float red[kWsumWarps][32];
    const size_t len = (size_t)cor * taps * cir, stride = (size_t)taps * cop * cip;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const size_t e = (size_t)blockIdx.x * 32 + lane;
    float s = 0.f;
    if (e < len) {
        const int ci = (int)(e % cir), tap = (int)((e / cir) % taps), co = (int)(e / ((size_t)cir * taps));
        const float* src = part + ((size_t)tap * cop + co) * cip + ci;
        float s0 = 0.f, s1 = 0.f;  // two chains: more loads in flight
        int p = w;
        for (; p + kWsumWarps < nparts; p += 2 * kWsumWarps) {
            s0 += src[(size_t)p * stride];
            s1 += src[(size_t)(p + kWsumWarps) * stride];
        }
        if (p < nparts)
            s0 += src[(size_t)p * stride];
        s = s0 + s1;
    }
    red[w][lane] = s;
    __syncthreads();
    if (w == 0 && e < len) {
        float t = 0.f;
#pragma unroll
        for (int k = 0; k < kWsumWarps; k++)
            t += red[k][lane];
        dw[e] = t;
    }
}

// column sums of a [count][C] bf16 tensor (C = 8, 16 or 32): per-block
// partials part[block][C].  Thread t reads 16-byte chunks (8 channels) of
// chunk column t % (C/8), four rows per iteration in flight; lanes of the
// same chunk column are summed by shuffles, then the warps in warp order.
__global__ void __launch_bounds__(256) k_colsum(const bf16* __restrict__ x, int C, size_t count,
                                                float* __restrict__ part)
{
    __shared__ float red[8][32];
    const int Q = C / 8;  // 16-byte chunks per row
    const int q = threadIdx.x % Q, rows = blockDim.x / Q, r0 = threadIdx.x / Q;
    const size_t stride = (size_t)gridDim.x * rows;
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    auto add = [&](const uint4& v) {
        const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float2 f = __bfloat1622float2(h[k]);
            acc[2 * k] += f.x;
            acc[2 * k + 1] += f.y;
        }
    };
    const uint4* x4 = reinterpret_cast<const uint4*>(x);
    size_t v = blockIdx.x * (size_t)rows + r0;
    for (; v + 3 * stride < count; v += 4 * stride) {
        const uint4 a0 = __ldg(x4 + v * Q + q), a1 = __ldg(x4 + (v + stride) * Q + q);
        const uint4 a2 = __ldg(x4 + (v + 2 * stride) * Q + q), a3 = __ldg(x4 + (v + 3 * stride) * Q + q);
        add(a0);
        add(a1);
        add(a2);
        add(a3);
    }
    for (; v < count; v += stride)
        add(__ldg(x4 + v * Q + q));
    // lanes l and l ^ o (o >= Q) hold the same chunk column
#pragma unroll
    for (int k = 0; k < 8; k++)
        for (int o = 16; o >= Q; o >>= 1)
            acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane < Q) {
#pragma unroll
        for (int k = 0; k < 8; k++)
            red[w][lane * 8 + k] = acc[k];
    }
    __syncthreads();
    if (threadIdx.x < C) {
        float t = 0.f;
        for (int s = 0; s < (int)(blockDim.x >> 5); s++)
            t += red[s][threadIdx.x];
        part[(size_t)blockIdx.x * C + threadIdx.x] = t;
    }
}

// ------------------------------------------------------------ loss

__device__ __forceinline__ size_t vidx(int box, int k, int j, int i, int n)
{
    return (((size_t)box * n + k) * n + j) * n + i;
}

// rf -> dout[0..4], rb = curl(E) - tb -> rb_out, per-block loss partials
__global__ void k_loss1(const float* __restrict__ out, const bf16* __restrict__ tgt, bf16* __restrict__ dout,
                        float* __restrict__ rb_out, float* __restrict__ lpart, int nb, int n, float gscale)
{
    __shared__ float red[32];
    const size_t nv = (size_t)nb * n * n * n;
    float ls = 0.f;
    for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < nv; v += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)((v / ((size_t)n * n)) % n);
        const int box = (int)(v / ((size_t)n * n * n));
        // the voxel's row: 8 FP32 outputs, 8 BF16 targets, 16 BF16 gradients (16-byte accesses)
        const float4 o0 = *reinterpret_cast<const float4*>(out + v * 8);
        const float4 o1 = *reinterpret_cast<const float4*>(out + v * 8 + 4);
        const uint4 t4 = *reinterpret_cast<const uint4*>(tgt + v * 8);
        const bf16* tg = reinterpret_cast<const bf16*>(&t4);
        const float o[8] = {o0.x, o0.y, o0.z, o0.w, o1.x, o1.y, o1.z, o1.w};
        __align__(16) bf16 d[16];
#pragma unroll
        for (int c = 0; c < 5; c++) {
            const float r = o[c] - __bfloat162float(tg[c]);
            ls += r * r;
            d[c] = __float2bfloat16_rn(gscale * r);
        }
#pragma unroll
        for (int c = 5; c < 16; c++)
            d[c] = __float2bfloat16_rn(0.f);
        uint4* d4 = reinterpret_cast<uint4*>(dout + v * 16);
        d4[0] = reinterpret_cast<const uint4*>(d)[0];
        d4[1] = reinterpret_cast<const uint4*>(d)[1];
        const float* oi = out + vidx(box, k, j, i + 1 == n ? 0 : i + 1, n) * 8;
        const float* oj = out + vidx(box, k, j + 1 == n ? 0 : j + 1, i, n) * 8;
        const float* ok = out + vidx(box, k + 1 == n ? 0 : k + 1, j, i, n) * 8;
        const float ex = o[5], ey = o[6], ez = o[7];
        const float dbx = -(oj[7] - ez) + (ok[6] - ey);
        const float dby = -(ok[5] - ex) + (oi[7] - ez);
        const float dbz = -(oi[6] - ey) + (oj[5] - ex);
        const float rx = dbx - __bfloat162float(tg[5]), ry = dby - __bfloat162float(tg[6]),
                    rz = dbz - __bfloat162float(tg[7]);
        ls += rx * rx + ry * ry + rz * rz;
        rb_out[v * 3] = rx;
        rb_out[v * 3 + 1] = ry;
        rb_out[v * 3 + 2] = rz;
    }
    ls = mhd_warp_sum(ls);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = ls;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++)
            s += red[w];
        lpart[blockIdx.x] = s;
    }
}

// dout[5..7] = gscale * curl^T(rb)
__global__ void k_loss2(const float* __restrict__ rb, bf16* __restrict__ dout, int nb, int n, float gscale)
{
    const size_t nv = (size_t)nb * n * n * n;
    for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < nv; v += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)((v / ((size_t)n * n)) % n);
        const int box = (int)(v / ((size_t)n * n * n));
        const float* r0 = rb + v * 3;
        const float* ri = rb + vidx(box, k, j, i == 0 ? n - 1 : i - 1, n) * 3;
        const float* rj = rb + vidx(box, k, j == 0 ? n - 1 : j - 1, i, n) * 3;
        const float* rk = rb + vidx(box, k == 0 ? n - 1 : k - 1, j, i, n) * 3;
        const float gx = r0[1] - rk[1] + rj[2] - r0[2];
        const float gy = rk[0] - r0[0] + r0[2] - ri[2];
        const float gz = r0[0] - rj[0] + ri[1] - r0[1];
        bf16* d = dout + v * 16;
        d[5] = __float2bfloat16_rn(gscale * gx);
        d[6] = __float2bfloat16_rn(gscale * gy);
        d[7] = __float2bfloat16_rn(gscale * gz);
    }
}

// ------------------------------------------------------------ state <-> features

// raw features (rho, mx, my, mz, E, Bx, By, Bz cell-centred) of one box;
// optional FP32 copy and optional standardised BF16 rows of 16 channels
__global__ void k_features(const float* __restrict__ u, const float* __restrict__ b, int n,
                           const float* __restrict__ mean, const float* __restrict__ inv_std,
                           float* __restrict__ raw, bf16* __restrict__ xo)
{
    const size_t nv = (size_t)n * n * n;
    for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < nv; v += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)(v / ((size_t)n * n));
        float f[8];
#pragma unroll
        for (int c = 0; c < 5; c++)
            f[c] = u[v * 5 + c];
        f[5] = 0.5f * (b[v * 3] + b[vidx(0, k, j, i + 1 == n ? 0 : i + 1, n) * 3]);
        f[6] = 0.5f * (b[v * 3 + 1] + b[vidx(0, k, j + 1 == n ? 0 : j + 1, i, n) * 3 + 1]);
        f[7] = 0.5f * (b[v * 3 + 2] + b[vidx(0, k + 1 == n ? 0 : k + 1, j, i, n) * 3 + 2]);
        if (raw)
#pragma unroll
            for (int c = 0; c < 8; c++)
                raw[v * 8 + c] = f[c];
        if (xo) {
            __align__(16) bf16 row[16];
#pragma unroll
            for (int c = 0; c < 8; c++)
                row[c] = __float2bfloat16_rn((f[c] - mean[c]) * inv_std[c]);
#pragma unroll
            for (int c = 8; c < 16; c++)
                row[c] = __float2bfloat16_rn(0.f);
            uint4* d = reinterpret_cast<uint4*>(xo + v * 16);
            d[0] = reinterpret_cast<const uint4*>(row)[0];
            d[1] = reinterpret_cast<const uint4*>(row)[1];
        }
    }
}

// y[v][c] = bf16((x[v][c] - mean[c]) * inv_std[c]) for c < C, zero for C <= c < CO
__global__ void k_normalize(const float* __restrict__ x, int C, size_t count, const float* __restrict__ mean,
                            const float* __restrict__ inv_std, bf16* __restrict__ y, int CO)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count * CO;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t v = e / CO;
        const int c = (int)(e - v * CO);
        y[e] = __float2bfloat16_rn(c < C ? (x[v * C + c] - mean[c]) * inv_std[c] : 0.f);
    }
}

// per-channel sums and sums of squares (FP64) of a [count][C] FP32 tensor
__global__ void k_moments(const float* __restrict__ x, int C, size_t count, double* __restrict__ sums)
{
    double s[16], q[16];
    for (int c = 0; c < C; c++)
        s[c] = q[c] = 0.0;
    for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < count; v += (size_t)gridDim.x * blockDim.x)
        for (int c = 0; c < C; c++) {
            const double a = x[v * C + c];
            s[c] += a;
            q[c] += a * a;
        }
    for (int c = 0; c < C; c++) {
        double a = s[c], bq = q[c];
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            bq += __shfl_xor_sync(0xffffffffu, bq, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&sums[c], a);
            atomicAdd(&sums[C + c], bq);
        }
    }
}

// coarse state = box filter of a fine one by f (cells: volume means; faces: means of f^2 fine faces)
__global__ void k_filter(const float* __restrict__ uf, const float* __restrict__ bfine, int nf, int f,
                         float* __restrict__ uc, float* __restrict__ bc)
{
    const int m = nf / f;
    const size_t nv = (size_t)m * m * m;
    const float inv3 = 1.0f / (float)(f * f * f), inv2 = 1.0f / (float)(f * f);
    for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < nv; v += (size_t)gridDim.x * blockDim.x) {
        const int I = (int)(v % m), J = (int)((v / m) % m), K = (int)(v / ((size_t)m * m));
        float s[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, bx = 0.f, by = 0.f, bz = 0.f;
        for (int dk = 0; dk < f; dk++)
            for (int dj = 0; dj < f; dj++)
                for (int di = 0; di < f; di++) {
                    const size_t c = vidx(0, K * f + dk, J * f + dj, I * f + di, nf);
#pragma unroll
                    for (int q = 0; q < 5; q++)
                        s[q] += uf[c * 5 + q];
                    if (di == 0)
                        bx += bfine[c * 3];
                    if (dj == 0)
                        by += bfine[c * 3 + 1];
                    if (dk == 0)
                        bz += bfine[c * 3 + 2];
                }
#pragma unroll
        for (int q = 0; q < 5; q++)
            uc[v * 5 + q] = s[q] * inv3;
        bc[v * 3] = bx * inv2;
        bc[v * 3 + 1] = by * inv2;
        bc[v * 3 + 2] = bz * inv2;
    }
}

// d[v] = (ua - ub, ba - bb) as 8 FP32 channels
__global__ void k_diff(const float* __restrict__ ua, const float* __restrict__ ba, const float* __restrict__ ub,
                       const float* __restrict__ bb, size_t nv, float* __restrict__ d)
{
    for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < nv; v += (size_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int q = 0; q < 5; q++)
            d[v * 8 + q] = ua[v * 5 + q] - ub[v * 5 + q];
#pragma unroll
        for (int q = 0; q < 3; q++)
            d[v * 8 + 5 + q] = ba[v * 3 + q] - bb[v * 3 + q];
    }
}

// ------------------------------------------------------------ correction step

// The correction follows a step of length 2 dt; none when that step was empty (dt at
// round-off: a run already at its final time).  dt may be absent (always correct).
__device__ __forceinline__ bool skip_step(const float* dt, float dt_min) { return dt && !(*dt > dt_min); }

// esum[2 + c] += sum over the box of out[.][c], c < 5 (the fluid corrections' means are removed,
// so the correction conserves mass, momentum and energy as the filtered fine step does)
__global__ void k_apply0(const float* __restrict__ out, size_t nv, double* __restrict__ esum,
                         const float* __restrict__ dt, float dt_min)
{
    if (skip_step(dt, dt_min))
        return;
    double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < nv; v += (size_t)gridDim.x * blockDim.x)
#pragma unroll
        for (int c = 0; c < 5; c++)
            s[c] += out[v * 8 + c];
#pragma unroll
    for (int c = 0; c < 5; c++) {
        const double t = mhd_warp_sum_d(s[c]);
        if ((threadIdx.x & 31) == 0)
            atomicAdd(&esum[2 + c], t);
    }
}

// candidate = state + alpha * correction (fluid part with its box mean removed) into (ut, bt);
// esum[0] += sum E, esum[1] += sum E of the candidate.  Nothing to do once an earlier attempt was
// committed (flags[1]).
__global__ void k_apply1(const float* __restrict__ u, const float* __restrict__ b, const float* __restrict__ out,
                         int n, const float* __restrict__ oscale, float bscale, float alpha, float* __restrict__ ut,
                         float* __restrict__ bt, double* __restrict__ esum, const int* __restrict__ flags,
                         const float* __restrict__ dt, float dt_min)
{
    if (flags[1] || skip_step(dt, dt_min))
        return;
    const size_t nv = (size_t)n * n * n;
    bscale *= alpha;
    float mean[5];
#pragma unroll
    for (int q = 0; q < 5; q++)
        mean[q] = (float)(esum[2 + q] / (double)nv);
    double e0 = 0.0, e1 = 0.0;
    for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < nv; v += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)(v / ((size_t)n * n));
        const float* o = out + v * 8;
        const float* oi = out + vidx(0, k, j, i + 1 == n ? 0 : i + 1, n) * 8;
        const float* oj = out + vidx(0, k, j + 1 == n ? 0 : j + 1, i, n) * 8;
        const float* ok = out + vidx(0, k + 1 == n ? 0 : k + 1, j, i, n) * 8;
#pragma unroll
        for (int q = 0; q < 5; q++)
            ut[v * 5 + q] = u[v * 5 + q] + alpha * oscale[q] * (o[q] - mean[q]);
        bt[v * 3] = b[v * 3] + bscale * (-(oj[7] - o[7]) + (ok[6] - o[6]));
        bt[v * 3 + 1] = b[v * 3 + 1] + bscale * (-(ok[5] - o[5]) + (oi[7] - o[7]));
        bt[v * 3 + 2] = b[v * 3 + 2] + bscale * (-(oi[6] - o[6]) + (oj[5] - o[5]));
        e0 += u[v * 5 + 4];
        e1 += ut[v * 5 + 4];
    }
    e0 = mhd_warp_sum_d(e0);
    e1 = mhd_warp_sum_d(e1);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&esum[0], e0);
        atomicAdd(&esum[1], e1);
    }
}

// positivity of the candidate (it needs the neighbours' candidate faces: a second pass)
__global__ void k_apply2(const float* __restrict__ ut, const float* __restrict__ bt, int n, int* __restrict__ flags,
                         const float* __restrict__ dt, float dt_min)
{
    if (flags[1] || skip_step(dt, dt_min))
        return;
    const size_t nv = (size_t)n * n * n;
    int bad = 0;
    for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < nv; v += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)(v / ((size_t)n * n));
        const float rho = ut[v * 5];
        const float bx = 0.5f * (bt[v * 3] + bt[vidx(0, k, j, i + 1 == n ? 0 : i + 1, n) * 3]);
        const float by = 0.5f * (bt[v * 3 + 1] + bt[vidx(0, k, j + 1 == n ? 0 : j + 1, i, n) * 3 + 1]);
        const float bz = 0.5f * (bt[v * 3 + 2] + bt[vidx(0, k + 1 == n ? 0 : k + 1, j, i, n) * 3 + 2]);
        const float mm = ut[v * 5 + 1] * ut[v * 5 + 1] + ut[v * 5 + 2] * ut[v * 5 + 2] + ut[v * 5 + 3] * ut[v * 5 + 3];
        const float p = (5.0f / 3.0f - 1.0f) * (ut[v * 5 + 4] - 0.5f * mm / rho - 0.5f * (bx * bx + by * by + bz * bz));
        if (!(rho > 0.f) || !(p > 0.f))
            bad = 1;
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0)
        atomicOr(flags, 1);
}

// commit the candidate unless a check failed (flags[1] = 1 once committed); the last attempt
// counts a fallback on the device when it fails too
__global__ void k_apply3(float* __restrict__ u, float* __restrict__ b, const float* __restrict__ ut,
                         const float* __restrict__ bt, size_t nv, int* __restrict__ flags,
                         const double* __restrict__ esum, float ecap, long long* __restrict__ fallbacks, int last,
                         const float* __restrict__ dt, float dt_min)
{
    if (flags[1] || skip_step(dt, dt_min))
        return;
    const bool energy_ok = fabs(esum[1] - esum[0]) <= (double)ecap * fabs(esum[0]);
    const bool ok = (flags[0] == 0) && energy_ok;
    if (blockIdx.x == 0 && threadIdx.x == 0 && !ok && last)
        atomicAdd(reinterpret_cast<unsigned long long*>(fallbacks), 1ULL);
    if (!ok)
        return;
    if (blockIdx.x == 0 && threadIdx.x == 0)
        atomicExch(&flags[2], 1);  // committed: read by the next attempt's kernels as flags[1]
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nv * 5; e += (size_t)gridDim.x * blockDim.x)
        u[e] = ut[e];
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nv * 3; e += (size_t)gridDim.x * blockDim.x)
        b[e] = bt[e];
}

// ------------------------------------------------------------ optimiser and weight packing

__global__ void k_adamw(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                        float* __restrict__ v, size_t count, float lr, float b1, float b2, float eps, float wd,
                        float c1, float c2)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x) {
        const float gg = g[e];
        const float mm = b1 * m[e] + (1.f - b1) * gg;
        const float vv = b2 * v[e] + (1.f - b2) * gg * gg;
        m[e] = mm;
        v[e] = vv;
        const float mh = mm / c1, vh = vv / c2;
        p[e] = p[e] - lr * (mh / (sqrtf(vh) + eps) + wd * p[e]);
    }
}

// master W[co][tap][ci] (FP32, ci < cir, co < cor) -> forward bf16 [cop][taps][cip] and
// data-gradient bf16 [cip][taps][cop] with the taps flipped (zeros in the padding)
__global__ void k_pack(const float* __restrict__ w, int cor, int cir, int taps, int cop, int cip,
                       bf16* __restrict__ wf, bf16* __restrict__ wd)
{
    const size_t tot = (size_t)cop * taps * cip;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
        const int ci = (int)(e % cip), tap = (int)((e / cip) % taps), co = (int)(e / ((size_t)cip * taps));
        const float x = (co < cor && ci < cir) ? w[((size_t)co * taps + tap) * cir + ci] : 0.f;
        if (wf)
            wf[e] = __float2bfloat16_rn(x);
        if (wd)
            wd[((size_t)ci * taps + (taps - 1 - tap)) * cop + co] = __float2bfloat16_rn(x);
    }
}

// ------------------------------------------------------------ host side

int g_sms = 0;
int sms()
{
    if (!g_sms) {
        int d = 0;
        cudaGetDevice(&d);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, d);
        if (g_sms <= 0)
            g_sms = 148;
    }
    return g_sms;
}

int st(cudaError_t e) { return e == cudaSuccess ? MHD_OK : MHD_ERR_CUDA; }

template <typename K>
cudaError_t set_smem(K kernel, size_t bytes)
{
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int CIN, int COUT, int KS, int EPI>
int launch_conv(const void* x, const void* w, const float* bias, void* y, void* zsave, const void* zprev, int nb,
                int n, cudaStream_t s)
{
    using HL = Halo<KS>;
    constexpr int TAPS = KS * KS * KS;
    const size_t smem = (size_t)HL::ROWS * row_bytes(CIN) + (size_t)COUT * (TAPS * CIN * 2 + 16);
    static bool attr = false;
    if (!attr) {
        if (set_smem(k_conv<CIN, COUT, KS, EPI>, smem) != cudaSuccess)
            return MHD_ERR_CUDA;
        attr = true;
    }
    const long long ntiles = (long long)nb * (n / TX) * (n / TY) * (n / TZ);
    const int per_sm = smem > 110 * 1024 ? 1 : 2;
    const long long grid = ntiles < (long long)sms() * per_sm * 2 ? ntiles : (long long)sms() * per_sm * 2;
    k_conv<CIN, COUT, KS, EPI><<<(unsigned)grid, 128, smem, s>>>(
        static_cast<const bf16*>(x), static_cast<const bf16*>(w), bias, y, static_cast<bf16*>(zsave),
        static_cast<const bf16*>(zprev), n, ntiles);
    return st(cudaGetLastError());
}

int* g_tc_err = nullptr;  // device error word of the tcgen05 kernels
bool g_tc_disabled = false;
bool g_tc_two_buffer = false;  // the single-loop two-buffer kernel in place of the warp-specialised one

unsigned short* g_gelu_tab = nullptr;  // gelu / gelu' tables of the warp-specialised convolution
float* g_grad_tab = nullptr;

template <int CIN, int COUT, int EPI>
int launch_conv_tc2(const void* x, const void* w, const float* bias, void* y, void* zsave, const void* zprev, int nb,
                    int n, cudaStream_t s)
{
    constexpr size_t smem = tc2_smem_bytes<CIN, COUT>();
    if (!g_gelu_tab) {  // once per process, ordered before the first use on this stream
        unsigned short* gt = nullptr;
        float* dt = nullptr;
        if (cudaMalloc(&gt, 65536 * sizeof(unsigned short)) != cudaSuccess ||
            cudaMalloc(&dt, 65536 * sizeof(float)) != cudaSuccess) {
            cudaFree(gt);
            return MHD_ERR_NOMEM;
        }
        k_gelu_tables<<<256, 256, 0, s>>>(gt, dt);
        // complete before any stream uses them (the first convolution is never captured:
        // a corrected step runs once uncaptured before its graph is built)
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
            return MHD_ERR_CUDA;
        g_gelu_tab = gt;
        g_grad_tab = dt;
    }
    static bool attr = false;
    if (!attr) {
        if (set_smem(k_conv_tc2<CIN, COUT, EPI>, smem) != cudaSuccess)
            return MHD_ERR_CUDA;
        attr = true;
    }
    const long long ntiles = (long long)nb * (n / TCX) * (n / TCY) * (n / TCZ);
    const long long grid = ntiles < (long long)sms() ? ntiles : (long long)sms();
    k_conv_tc2<CIN, COUT, EPI><<<(unsigned)grid, kTc2Warps * 32, smem, s>>>(
        static_cast<const bf16*>(x), static_cast<const bf16*>(w), bias, y, static_cast<bf16*>(zsave),
        static_cast<const bf16*>(zprev), n, ntiles, g_tc_err, g_gelu_tab, g_grad_tab);
    return st(cudaGetLastError());
}

template <int CIN, int COUT, int EPI>
int launch_conv_tc(const void* x, const void* w, const float* bias, void* y, void* zsave, const void* zprev, int nb,
                   int n, cudaStream_t s)
{
    if (!g_tc_err && cudaMalloc(&g_tc_err, sizeof(int)) == cudaSuccess)
        cudaMemset(g_tc_err, 0, sizeof(int));
    if (!g_tc_err)
        return MHD_ERR_NOMEM;
    if (!g_tc_two_buffer)
        return launch_conv_tc2<CIN, COUT, EPI>(x, w, bias, y, zsave, zprev, nb, n, s);
    const size_t smem = 2 * (size_t)(CIN / 8) * kChunkBytes + (size_t)27 * (CIN / 8) * COUT * 16;  // A x 2, W
    static bool attr = false;
    if (!attr) {
        if (set_smem(k_conv_tc<CIN, COUT, EPI>, smem) != cudaSuccess)
            return MHD_ERR_CUDA;
        attr = true;
    }
    if (!g_tc_err && cudaMalloc(&g_tc_err, sizeof(int)) == cudaSuccess)
        cudaMemset(g_tc_err, 0, sizeof(int));
    if (!g_tc_err)
        return MHD_ERR_NOMEM;
    const long long ntiles = (long long)nb * (n / TCX) * (n / TCY) * (n / TCZ);
    const long long grid = ntiles < (long long)sms() ? ntiles : (long long)sms();
    k_conv_tc<CIN, COUT, EPI><<<(unsigned)grid, 256, smem, s>>>(
        static_cast<const bf16*>(x), static_cast<const bf16*>(w), bias, y, static_cast<bf16*>(zsave),
        static_cast<const bf16*>(zprev), n, ntiles, g_tc_err);
    return st(cudaGetLastError());
}

bool use_tc(int n) { return !g_tc_disabled && n % TCX == 0 && n % TCY == 0 && n % TCZ == 0; }

template <int CIN, int COUTP, int KS>
size_t wgrad_parts(int nb, int n)
{
    using S = WgradShape<CIN, COUTP, KS>;
    const long long ntiles = (long long)nb * (n / TX) * (n / TY) * (n / TZ);
    const long long grid = ntiles < (long long)sms() * 2 ? ntiles : (long long)sms() * 2;
    return (size_t)grid * S::WK;
}

template <int CIN, int COUTP, int KS>
int launch_wgrad(const void* a, const void* dz, float* part, float* dw, int cor, int cir, int nb, int n,
                 cudaStream_t s)
{
    using S = WgradShape<CIN, COUTP, KS>;
    using HL = Halo<KS>;
    const size_t smem = (size_t)HL::ROWS * row_bytes(CIN) + (size_t)TV * row_bytes(COUTP);
    static bool attr = false;
    if (!attr) {
        if (set_smem(k_wgrad<CIN, COUTP, KS>, smem) != cudaSuccess)
            return MHD_ERR_CUDA;
        attr = true;
    }
    const long long ntiles = (long long)nb * (n / TX) * (n / TY) * (n / TZ);
    const long long grid = ntiles < (long long)sms() * 2 ? ntiles : (long long)sms() * 2;
    k_wgrad<CIN, COUTP, KS><<<(unsigned)grid, S::THREADS, smem, s>>>(static_cast<const bf16*>(a),
                                                                      static_cast<const bf16*>(dz), part, n, ntiles);
    if (cudaGetLastError() != cudaSuccess)
        return MHD_ERR_CUDA;
    const size_t len = (size_t)cor * S::TAPS * cir;
    k_wsum<<<(unsigned)((len + 31) / 32), kWsumWarps * 32, 0, s>>>(part, (int)(grid * S::WK), S::TAPS, COUTP, CIN,
                                                                    cor, cir, dw);
    return st(cudaGetLastError());
}

bool shape_ok(int nb, int n) { return nb > 0 && n >= 8 && n % 8 == 0 && n <= 1024; }

unsigned blocks_for(size_t work, int threads)
{
    size_t b = (work + threads - 1) / threads;
    const size_t cap = (size_t)sms() * 8;
    return (unsigned)(b < cap ? (b ? b : 1) : cap);
}

}  // namespace

// ------------------------------------------------------------ C ABI

extern "C" MHD_API int mhd_cl_conv(int kind, const void* x, const void* w, const float* bias, void* y, void* zsave,
                                   const void* zprev, int nb, int n, void* stream)
{
    if (!x || !w || !y || !shape_ok(nb, n))
        return MHD_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (kind) {
    case MHD_CL_FWD_IN:
        if (!bias || !zsave)
            return MHD_ERR_ARG;
        return use_tc(n) ? launch_conv_tc<16, 32, EPI_GELU>(x, w, bias, y, zsave, nullptr, nb, n, s)
                         : launch_conv<16, 32, 3, EPI_GELU>(x, w, bias, y, zsave, nullptr, nb, n, s);
    case MHD_CL_FWD_HID:
        if (!bias || !zsave)
            return MHD_ERR_ARG;
        return use_tc(n) ? launch_conv_tc<32, 32, EPI_GELU>(x, w, bias, y, zsave, nullptr, nb, n, s)
                         : launch_conv<32, 32, 3, EPI_GELU>(x, w, bias, y, zsave, nullptr, nb, n, s);
    case MHD_CL_FWD_HEAD:
        return bias ? launch_conv<32, 8, 1, EPI_LINEAR_F32>(x, w, bias, y, nullptr, nullptr, nb, n, s) : MHD_ERR_ARG;
    case MHD_CL_DGRAD_HEAD:
        return zprev ? launch_conv<16, 32, 1, EPI_DGRAD>(x, w, nullptr, y, nullptr, zprev, nb, n, s) : MHD_ERR_ARG;
    case MHD_CL_DGRAD_HID:
        if (!zprev)
            return MHD_ERR_ARG;
        return use_tc(n) ? launch_conv_tc<32, 32, EPI_DGRAD>(x, w, nullptr, y, nullptr, zprev, nb, n, s)
                         : launch_conv<32, 32, 3, EPI_DGRAD>(x, w, nullptr, y, nullptr, zprev, nb, n, s);
    }
    return MHD_ERR_ARG;
}

// 1: the 3^3 convolutions of edges that are multiples of 16 run on tcgen05 (the default); 0: the
// mma.sync kernels everywhere.  Returns the previous setting.
extern "C" MHD_API int mhd_cl_use_tcgen05(int enable)
{
    const int prev = g_tc_disabled ? 0 : (g_tc_two_buffer ? 2 : 1);
    g_tc_disabled = (enable == 0);
    g_tc_two_buffer = (enable == 2);
    return prev;
}

// Error bits of the tcgen05 kernels' bounded waits (DEVERR_TIMEOUT), cleared by the read.
extern "C" MHD_API int mhd_cl_device_errors(void)
{
    if (!g_tc_err)
        return 0;
    int h = 0;
    if (cudaMemcpy(&h, g_tc_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return -1;
    cudaMemset(g_tc_err, 0, sizeof(int));
    return h;
}

extern "C" MHD_API long long mhd_cl_wgrad_scratch(int kind, int nb, int n)
{
    if (!shape_ok(nb, n))
        return -1;
    switch (kind) {
    case MHD_CL_WG_IN: return (long long)(wgrad_parts<16, 32, 3>(nb, n) * 27 * 32 * 16 * sizeof(float));
    case MHD_CL_WG_HID: return (long long)(wgrad_parts<32, 32, 3>(nb, n) * 27 * 32 * 32 * sizeof(float));
    case MHD_CL_WG_HEAD: return (long long)(wgrad_parts<32, 16, 1>(nb, n) * 1 * 16 * 32 * sizeof(float));
    }
    return -1;
}

extern "C" MHD_API int mhd_cl_wgrad(int kind, const void* a, const void* dz, float* scratch, float* dw, int nb, int n,
                                    void* stream)
{
    if (!a || !dz || !scratch || !dw || !shape_ok(nb, n))
        return MHD_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (kind) {
    case MHD_CL_WG_IN: return launch_wgrad<16, 32, 3>(a, dz, scratch, dw, 32, 8, nb, n, s);
    case MHD_CL_WG_HID: return launch_wgrad<32, 32, 3>(a, dz, scratch, dw, 32, 32, nb, n, s);
    case MHD_CL_WG_HEAD: return launch_wgrad<32, 16, 1>(a, dz, scratch, dw, 8, 32, nb, n, s);
    }
    return MHD_ERR_ARG;
}

extern "C" MHD_API int mhd_cl_colsum(const void* x, int channels, long long count, int nout, float* scratch,
                                     float* out, void* stream)
{
    if (!x || !scratch || !out || count <= 0 || (channels != 8 && channels != 16 && channels != 32) || nout <= 0 ||
        nout > channels)
        return MHD_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int threads = 256, blocks = 256;  // blocks: the scratch holds 256 * channels partials
    if (reinterpret_cast<uintptr_t>(x) & 15)
        return MHD_ERR_ARG;  // rows are read as 16-byte chunks
    k_colsum<<<blocks, threads, 0, s>>>(static_cast<const bf16*>(x), channels, (size_t)count, scratch);
    if (cudaGetLastError() != cudaSuccess)
        return MHD_ERR_CUDA;
    k_sum_parts<<<(unsigned)((nout + 31) / 32), kSumWarps * 32, 0, s>>>(scratch, blocks, (size_t)channels,
                                                                        (size_t)nout, out);
    return st(cudaGetLastError());
}

extern "C" MHD_API int mhd_cl_loss(const float* out, const void* target, void* dout, float* rb_scratch,
                                   float* loss_scratch, float* loss, int nb, int n, void* stream)
{
    if (!out || !target || !dout || !rb_scratch || !loss_scratch || !loss || !shape_ok(nb, n))
        return MHD_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(out) | reinterpret_cast<uintptr_t>(target) | reinterpret_cast<uintptr_t>(dout)) &
        15)
        return MHD_ERR_ARG;  // rows are moved in 16-byte pieces
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t nv = (size_t)nb * n * n * n;
    const float gscale = 2.0f / (8.0f * (float)nv);
    const unsigned blocks = 512;
    k_loss1<<<blocks, 256, 0, s>>>(out, static_cast<const bf16*>(target), static_cast<bf16*>(dout), rb_scratch,
                                   loss_scratch, nb, n, gscale);
    if (cudaGetLastError() != cudaSuccess)
        return MHD_ERR_CUDA;
    k_loss2<<<blocks_for(nv, 256), 256, 0, s>>>(rb_scratch, static_cast<bf16*>(dout), nb, n, gscale);
    if (cudaGetLastError() != cudaSuccess)
        return MHD_ERR_CUDA;
    k_sum_parts<<<1, kSumWarps * 32, 0, s>>>(loss_scratch, (int)blocks, 1, 1, loss);  // sum of squares; /(8N) on the host
    return st(cudaGetLastError());
}

extern "C" MHD_API int mhd_cl_features(const float* u, const float* b, int n, const float* mean,
                                       const float* inv_std, float* raw, void* x, void* stream)
{
    if (!u || !b || n <= 0 || (!raw && !x) || (x && (!mean || !inv_std)))
        return MHD_ERR_ARG;
    const size_t nv = (size_t)n * n * n;
    k_features<<<blocks_for(nv, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(u, b, n, mean, inv_std, raw,
                                                                                   static_cast<bf16*>(x));
    return st(cudaGetLastError());
}

extern "C" MHD_API int mhd_cl_normalize(const float* x, int channels, long long count, const float* mean,
                                        const float* inv_std, void* y, int out_channels, void* stream)
{
    if (!x || !mean || !inv_std || !y || channels <= 0 || out_channels < channels || count <= 0)
        return MHD_ERR_ARG;
    k_normalize<<<blocks_for((size_t)count * out_channels, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        x, channels, (size_t)count, mean, inv_std, static_cast<bf16*>(y), out_channels);
    return st(cudaGetLastError());
}

extern "C" MHD_API int mhd_cl_moments(const float* x, int channels, long long count, double* sums, void* stream)
{
    if (!x || !sums || channels <= 0 || channels > 16 || count <= 0)
        return MHD_ERR_ARG;
    k_moments<<<blocks_for((size_t)count, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(x, channels,
                                                                                              (size_t)count, sums);
    return st(cudaGetLastError());
}

extern "C" MHD_API int mhd_cl_filter(const float* u_fine, const float* b_fine, int n_fine, int factor, float* u_coarse,
                                     float* b_coarse, void* stream)
{
    if (!u_fine || !b_fine || !u_coarse || !b_coarse || factor <= 0 || n_fine <= 0 || n_fine % factor)
        return MHD_ERR_ARG;
    const int m = n_fine / factor;
    k_filter<<<blocks_for((size_t)m * m * m, 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
        u_fine, b_fine, n_fine, factor, u_coarse, b_coarse);
    return st(cudaGetLastError());
}

extern "C" MHD_API int mhd_cl_diff(const float* ua, const float* ba, const float* ub, const float* bb, int n, float* d,
                                   void* stream)
{
    if (!ua || !ba || !ub || !bb || !d || n <= 0)
        return MHD_ERR_ARG;
    const size_t nv = (size_t)n * n * n;
    k_diff<<<blocks_for(nv, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(ua, ba, ub, bb, nv, d);
    return st(cudaGetLastError());
}

// between attempts: committed -> flags[1]; clear the failure bit and the energy sums
__global__ void k_apply_next(int* flags, double* esum)
{
    flags[1] = flags[2];
    flags[0] = 0;
    esum[0] = esum[1] = 0.0;
}

extern "C" MHD_API int mhd_cl_apply(float* u, float* b, const float* out, int n, const float* oscale, float bscale,
                                    float* u_tmp, float* b_tmp, int* flags, double* esum, float ecap,
                                    long long* fallbacks, const float* dt, float dt_min, void* stream)
{
    const float alphas[3] = {1.0f, 0.5f, 0.25f};
    if (!u || !b || !out || !oscale || !u_tmp || !b_tmp || !flags || !esum || !fallbacks || n <= 0)
        return MHD_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t nv = (size_t)n * n * n;
    if (cudaMemsetAsync(flags, 0, 4 * sizeof(int), s) != cudaSuccess ||
        cudaMemsetAsync(esum, 0, 8 * sizeof(double), s) != cudaSuccess)
        return MHD_ERR_CUDA;
    const unsigned blocks = blocks_for(nv, 256);
    k_apply0<<<blocks, 256, 0, s>>>(out, nv, esum, dt, dt_min);
    for (int a = 0; a < 3; a++) {  // the full correction, else half, else a quarter, else none
        if (a)
            k_apply_next<<<1, 1, 0, s>>>(flags, esum);
        k_apply1<<<blocks, 256, 0, s>>>(u, b, out, n, oscale, bscale, alphas[a], u_tmp, b_tmp, esum, flags, dt,
                                        dt_min);
        k_apply2<<<blocks, 256, 0, s>>>(u_tmp, b_tmp, n, flags, dt, dt_min);
        k_apply3<<<blocks, 256, 0, s>>>(u, b, u_tmp, b_tmp, nv, flags, esum, ecap, fallbacks, a == 2, dt, dt_min);
    }
    return st(cudaGetLastError());
}

extern "C" MHD_API int mhd_cl_adamw(float* p, const float* g, float* m, float* v, long long count, int step, float lr,
                                    float beta1, float beta2, float eps, float wd, void* stream)
{
    if (!p || !g || !m || !v || count <= 0 || step <= 0)
        return MHD_ERR_ARG;
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    k_adamw<<<blocks_for((size_t)count, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        p, g, m, v, (size_t)count, lr, beta1, beta2, eps, wd, c1, c2);
    return st(cudaGetLastError());
}

extern "C" MHD_API int mhd_cl_pack(const float* w, int cout_real, int cin_real, int taps, int cout_pad, int cin_pad,
                                   void* w_fwd, void* w_dgrad, void* stream)
{
    if (!w || cout_real <= 0 || cin_real <= 0 || taps <= 0 || cout_pad < cout_real || cin_pad < cin_real ||
        (!w_fwd && !w_dgrad))
        return MHD_ERR_ARG;
    const size_t tot = (size_t)cout_pad * taps * cin_pad;
    k_pack<<<blocks_for(tot, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        w, cout_real, cin_real, taps, cout_pad, cin_pad, static_cast<bf16*>(w_fwd), static_cast<bf16*>(w_dgrad));
    return st(cudaGetLastError());
}
