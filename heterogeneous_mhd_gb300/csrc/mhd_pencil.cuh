// Pencil engine: a pencil of n cells is owned by T = n/C threads, thread t
// holding the C consecutive cells t*C .. t*C+C-1 in registers.  Neighbour
// values across chunk boundaries move by warp shuffles; when a pencil spans
// several warps (T > 32) the values at the warp seams go through shared
// memory with one block barrier per exchange round.  The periodic wrap
// (cell n-1 <-> cell 0) is the wrap of the thread index.
#pragma once
#include <cuda_runtime.h>

namespace mhd {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kSeamVals = 10;  // largest exchange (values per thread and round)

// Contiguous chunk of NF values to/from shared memory; 128-bit accesses for
// float when NF % 4 == 0 (the caller guarantees 16-byte alignment).
// component of the untransposed state that the sweep along axis AX sees as
// its component s: u (rho, m_d, m_j, m_k, E), b (b_d, b_j, b_k) with
// (d, j, k) = (x, y, z), (y, x, z), (z, x, y)
template <int AX>
__host__ __device__ constexpr int sweep_u(int s)
{
    return AX == 0 ? s : (AX == 1 ? (s == 1 ? 2 : (s == 2 ? 1 : s)) : (s == 1 ? 3 : (s == 2 ? 1 : (s == 3 ? 2 : s))));
}
template <int AX>
__host__ __device__ constexpr int sweep_b(int s)
{
    return AX == 0 ? s : (AX == 1 ? (s == 0 ? 1 : (s == 1 ? 0 : 2)) : (s == 0 ? 2 : (s == 1 ? 0 : 1)));
}

// linear cell of (position i along the sweep, x, plane k) for AX = 1 (k = z) and AX = 2 (k = y)
template <int AX>
__device__ __forceinline__ size_t sweep_cell(int i, int x, int k, int nx, int ny)
{
    return AX == 1 ? ((size_t)k * ny + i) * nx + x : ((size_t)i * ny + k) * nx + x;
}

// Walks the elements e = start, start + step, ... of a tile of rows of W
// elements as (row, w) without a division per element.
struct RowIter {
    int row, w, drow, dw, W;
    __device__ __forceinline__ RowIter(int start, int step, int W_) : W(W_)
    {
        row = start / W;
        w = start - row * W;
        drow = step / W;
        dw = step - drow * W;
    }
    __device__ __forceinline__ void next()
    {
        row += drow;
        w += dw;
        if (w >= W) {
            w -= W;
            row++;
        }
    }
};

// Gather an n-row tile into pencil-major shared memory: row r of the tile is
// W = pencils x NC consecutive words at src_row0 + r * rstride (pencil p of
// the row starting at word col(p) * NC of it), and word (p, c) of row r goes
// to dst[p * PS + r * NC + c].  Each thread owns one fixed column w of the
// tile and walks the rows, so an element costs one 4-byte cp.async and two
// pointer increments; consecutive threads read consecutive words.
template <int NC, typename Col>
__device__ __forceinline__ void gather_tile(float* dst, int PS, const float* src_row0, size_t rstride, int pencils,
                                            int n, Col col, int tid, int nt)
{
    const int W = pencils * NC, rpp = nt / W;
    if (rpp == 0) {  // fewer threads than columns: a thread walks several columns
        for (int w = tid; w < W; w += nt) {
            const int p = w / NC, c = w - p * NC;
            for (int r = 0; r < n; r++)
                cp_async4(dst + p * PS + r * NC + c, src_row0 + (size_t)col(p) * NC + c + (size_t)r * rstride);
        }
        return;
    }
    if (tid >= rpp * W)
        return;
    const int w = tid % W, r0 = tid / W;
    const int p = w / NC, c = w - p * NC;
    float* d = dst + p * PS + r0 * NC + c;
    const float* s = src_row0 + (size_t)col(p) * NC + c + (size_t)r0 * rstride;
    const size_t sstep = (size_t)rpp * rstride;
    for (int r = r0; r < n; r += rpp, d += rpp * NC, s += sstep)
        cp_async4(d, s);
}

// The inverse: row r of a pencil-major shared tile back to its global row.
template <int NC>
__device__ __forceinline__ void scatter_tile(float* dst_row0, size_t rstride, const float* src, int PS, int pencils,
                                             int n, int tid, int nt)
{
    const int W = pencils * NC, rpp = nt / W;
    if (rpp == 0) {
        for (int w = tid; w < W; w += nt) {
            const int p = w / NC, c = w - p * NC;
            for (int r = 0; r < n; r++)
                dst_row0[w + (size_t)r * rstride] = src[p * PS + r * NC + c];
        }
        return;
    }
    if (tid >= rpp * W)
        return;
    const int w = tid % W, r0 = tid / W;
    const int p = w / NC, c = w - p * NC;
    const float* s = src + p * PS + r0 * NC + c;
    float* d = dst_row0 + w + (size_t)r0 * rstride;
    const size_t dstep = (size_t)rpp * rstride;
    for (int r = r0; r < n; r += rpp, s += rpp * NC, d += dstep)
        *d = *s;
}

// padding (elements) of the pencil stride of tiles that the y/z sweeps fill
// element by element: keeps the shared stores of a warp within 2-way conflicts
constexpr int kSweepPad = 8;

// Global chunk loads/stores of NF consecutive values with the widest vector
// the alignment allows (the caller guarantees it: 16 B for NF % 4 == 0, 8 B
// for NF % 2 == 0).
template <typename R, int NF>
__device__ __forceinline__ void ldg_chunk(const R* src, R (&dst)[NF])
{
    if constexpr (sizeof(R) == 4 && NF % 4 == 0) {
        const float4* s4 = reinterpret_cast<const float4*>(src);
#pragma unroll
        for (int v = 0; v < NF / 4; v++) {
            const float4 x = __ldg(s4 + v);
            dst[4 * v] = x.x;
            dst[4 * v + 1] = x.y;
            dst[4 * v + 2] = x.z;
            dst[4 * v + 3] = x.w;
        }
    } else if constexpr (sizeof(R) == 4 && NF % 2 == 0) {
        const float2* s2 = reinterpret_cast<const float2*>(src);
#pragma unroll
        for (int v = 0; v < NF / 2; v++) {
            const float2 x = __ldg(s2 + v);
            dst[2 * v] = x.x;
            dst[2 * v + 1] = x.y;
        }
    } else {
#pragma unroll
        for (int v = 0; v < NF; v++)
            dst[v] = src[v];
    }
}

template <typename R, int NF>
__device__ __forceinline__ void stg_chunk(R* dst, const R (&src)[NF])
{
    if constexpr (sizeof(R) == 4 && NF % 4 == 0) {
        float4* d4 = reinterpret_cast<float4*>(dst);
#pragma unroll
        for (int v = 0; v < NF / 4; v++)
            d4[v] = make_float4(src[4 * v], src[4 * v + 1], src[4 * v + 2], src[4 * v + 3]);
    } else if constexpr (sizeof(R) == 4 && NF % 2 == 0) {
        float2* d2 = reinterpret_cast<float2*>(dst);
#pragma unroll
        for (int v = 0; v < NF / 2; v++)
            d2[v] = make_float2(src[2 * v], src[2 * v + 1]);
    } else {
#pragma unroll
        for (int v = 0; v < NF; v++)
            dst[v] = src[v];
    }
}

template <typename R, int NF>
__device__ __forceinline__ void lds_chunk(const R* src, R (&dst)[NF])
{
    if constexpr (sizeof(R) == 4 && NF % 4 == 0) {
        const float4* s4 = reinterpret_cast<const float4*>(src);
#pragma unroll
        for (int v = 0; v < NF / 4; v++) {
            const float4 x = s4[v];
            dst[4 * v] = x.x;
            dst[4 * v + 1] = x.y;
            dst[4 * v + 2] = x.z;
            dst[4 * v + 3] = x.w;
        }
    } else {
#pragma unroll
        for (int v = 0; v < NF; v++)
            dst[v] = src[v];
    }
}

template <typename R, int NF>
__device__ __forceinline__ void sts_chunk(R* dst, const R (&src)[NF])
{
    if constexpr (sizeof(R) == 4 && NF % 4 == 0) {
        float4* d4 = reinterpret_cast<float4*>(dst);
#pragma unroll
        for (int v = 0; v < NF / 4; v++)
            d4[v] = make_float4(src[4 * v], src[4 * v + 1], src[4 * v + 2], src[4 * v + 3]);
    } else {
#pragma unroll
        for (int v = 0; v < NF; v++)
            dst[v] = src[v];
    }
}

// Exchange helper for one group of T threads (T a power of two <= 32, or a
// multiple of 32).  `seam` is this CTA's scratch for warp-seam values: two
// alternating banks of [warps][kSeamVals] elements.
template <typename R, int T, bool kNamed = false>
struct Group {
    static constexpr bool kMulti = (T > 32);
    static constexpr int kWarps = kMulti ? T / 32 : 1;
    static_assert(T <= 32 ? ((T & (T - 1)) == 0) : (T % 32 == 0), "T must be a power of two <= 32 or a multiple of 32");

    int t;       // thread index inside the group (0..T-1)
    int lane;    // lane in the warp
    int warp;    // warp index in the CTA
    int gwarp0;  // first warp of this group in the CTA

    __device__ __forceinline__ Group(int tid)
    {
        t = tid % T;
        lane = tid & 31;
        warp = tid >> 5;
        gwarp0 = warp - (t >> 5);
    }

    // kNamed: the barrier of this group's T threads only (named barrier 1 + group
    // index; 0 is __syncthreads'), so that the row groups of a CTA do not wait for
    // one another; otherwise the CTA barrier (a CTA that is one group).
    __device__ __forceinline__ void sync() const
    {
        if constexpr (kNamed) {
            __syncwarp();
            asm volatile("barrier.sync %0, %1;" ::"r"(1 + gwarp0 / kWarps), "r"(T) : "memory");
        } else {
            __syncthreads();
        }
    }

    // Max over the group's values (starting from 0, NaN skipped as by fmax).
    __device__ __forceinline__ R max(R x, R* red) const
    {
        const int w = (T < 32) ? T : 32;
#pragma unroll
        for (int o = w / 2; o > 0; o >>= 1)
            x = fmax(x, __shfl_xor_sync(kFull, x, o));
        if constexpr (kMulti) {
            if (lane == 0)
                red[warp] = x;
            sync();
            R m = R(0);
#pragma unroll
            for (int s = 0; s < kWarps; s++)
                m = fmax(m, red[gwarp0 + s]);
            return m;
        } else {
            return fmax(R(0), x);
        }
    }

    // out[k] = x[k] of the thread t+1 (dir = +1) or t-1 (dir = -1), periodic.
    // For T > 32 one barrier; `bank` (0/1) must alternate between consecutive calls.
    template <int K>
    __device__ __forceinline__ void shift(const R (&x)[K], R (&out)[K], int dir, R* seam, int bank) const
    {
        if constexpr (!kMulti) {
            const int src = (dir > 0) ? ((t + 1) & (T - 1)) : ((t + T - 1) & (T - 1));
#pragma unroll
            for (int k = 0; k < K; k++)
                out[k] = __shfl_sync(kFull, x[k], src, T);
        } else {
            static_assert(K <= kSeamVals, "too many values per exchange");
            R* s = seam + bank * (32 * kSeamVals);  // [warp][kSeamVals]: slots independent of K
            const int edge = (dir > 0) ? 0 : 31;     // the lane whose value crosses the seam
            if (lane == edge) {
#pragma unroll
                for (int k = 0; k < K; k++)
                    s[warp * kSeamVals + k] = x[k];
            }
#pragma unroll
            for (int k = 0; k < K; k++)
                out[k] = (dir > 0) ? __shfl_down_sync(kFull, x[k], 1) : __shfl_up_sync(kFull, x[k], 1);
            sync();
            const int need = (dir > 0) ? 31 : 0;
            if (lane == need) {
                const int gw = warp - gwarp0;
                const int nb = (dir > 0) ? ((gw + 1) % kWarps) : ((gw + kWarps - 1) % kWarps);
#pragma unroll
                for (int k = 0; k < K; k++)
                    out[k] = s[(gwarp0 + nb) * kSeamVals + k];
            }
        }
    }
};

}  // namespace mhd
