// Launcher bodies shared by the kernel-set translation units.  Included once
// per unit with MHD_SET_NAME, MHD_REAL and MHD_EXACT defined.
//
// Each operator has a register-resident kernel for the common pencil lengths
// (fluidx: n = 4T with T in {8..128} or 3T with T in {16..128}; advectbyzx:
// n = 8T, T in {4..64} or 6T, T in {8..64}; transposes: full 32x32 tiles, or
// 16x16 tiles for edges that are multiples of 16) and a general kernel for
// every other shape.  FP64 uses the general kernels.  The batch's work-list
// launches (one launch per operator over several size classes) are at the end.
#include "mhd_advect2.cuh"
#include "mhd_advect3.cuh"
#include "mhd_advect4.cuh"
#include "mhd_advect5.cuh"
#include "mhd_advect6.cuh"
#include "mhd_fluidx2.cuh"
#include "mhd_launch.h"
#include "mhd_multi.cuh"
#include "mhd_tmap.h"
#include "mhd_transpose2.cuh"
#include "mhd_transpose3.cuh"

namespace mhd {
namespace MHD_SET_NAME {

using R = MHD_REAL;
constexpr bool EX = MHD_EXACT;
constexpr bool kV2 = (sizeof(R) == 4);

// Raise a kernel's dynamic shared-memory limit to the device's opt-in maximum
// minus its static shared memory (once per kernel).  Kernels that stage all
// their input by TMA ask for the largest shared-memory carveout (they do not
// use L1 for data), so residency is set by registers and shared memory only.
template <typename K>
static cudaError_t allow_smem(K kernel, bool& done, bool tma_staged = false)
{
    if (done)
        return cudaSuccess;
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    if (e == cudaSuccess)
        e = cudaFuncGetAttributes(&fa, kernel);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
    if (e == cudaSuccess && tma_staged)
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e == cudaSuccess)
        done = true;
    return e;
}

// devices whose occupancy figures the persistent launchers cache
constexpr int kMaxOccDevices = 64;

static bool pow2_in(int T, int lo, int hi) { return T >= lo && T <= hi && (T & (T - 1)) == 0; }

// ------------------------------------------------------------------ fluidx

struct FxPlan {
    int C, T, P;  // C == 0: general kernel with P pencils per CTA
};

static FxPlan plan_fluidx(int nx, int ny, bool aligned)
{
    FxPlan p{0, 0, 0};
    if (kV2 && aligned) {
        if (tune_value(TUNE_FLUIDX_C) == 8 && nx % 8 == 0 && pow2_in(nx / 8, 8, 64))
            p.C = 8, p.T = nx / 8;
        else if (nx % 4 == 0 && pow2_in(nx / 4, 8, 128))
            p.C = 4, p.T = nx / 4;
        else if (nx % 3 == 0 && nx % 4 == 0 && pow2_in(nx / 3, 16, 128))
            p.C = 3, p.T = nx / 3;
        if (p.C) {
            int target = tune_value(TUNE_FLUIDX_THREADS);
            if (target != 32 && target != 64 && target != 128 && target != 256)
                target = 64;  // measured best on GB300 at 256^3 (autotune.py)
            p.P = 0;
            for (int P = 1; P <= ny; P++)
                if (ny % P == 0 && P * p.T <= (target > p.T ? target : p.T) && (P * p.T) % 32 == 0 && P * p.T <= 256)
                    p.P = P;
            if (p.P)
                return p;
        }
    }
    p.C = p.T = 0;
    p.P = fluidx_pencils(nx, ny);
    return p;
}

template <int C, int T, int AX = 0>
static cudaError_t launch_fx2(const FluidxArgs& a, cudaStream_t s)
{
    static bool attr = false;
    cudaError_t e = allow_smem(k_fluidx2<R, EX, C, T, AX>, attr, true);
    if (e != cudaSuccess)
        return e;
    // grid: (pencil groups along j, planes along k (a range along z: kcount), boxes)
    const int nj = (AX == 0) ? a.ny : a.nx, nk = (AX == 2) ? a.ny : (a.kcount ? a.kcount : a.nz);
    dim3 grid(nj / a.P, nk, a.bs.count);
    SweepMaps tm{};
    size_t smem = fluidx2_smem_elems(C * T, a.P) * sizeof(R);
    if constexpr (AX != 0) {
        // the x-major state as (5 nx words, ny, nz) for u and (3 nx, ny, nz) for b;
        // boxes of P cells along x by the pencil along y (AX 1) or z (AX 2), in
        // boxes of at most 256 rows
        constexpr int n = C * T, rows = (n + 255) / 256 > 1 ? n / ((n + 255) / 256) : n;
        const uint32_t by = (AX == 1) ? rows : 1, bz = (AX == 1) ? 1 : rows;
        const uint64_t ny = a.ny, nz = a.nz;
        e = encode_map_3d(&tm.u_in, a.uu, 5ull * a.nx, ny, nz, 5 * kSweepP, by, bz);
        if (e == cudaSuccess)
            e = encode_map_3d(&tm.b_in, a.ub, 3ull * a.nx, ny, nz, 3 * kSweepP, by, bz);
        if (e == cudaSuccess)
            e = encode_map_3d(&tm.bn_in, a.ub, 3ull * a.nx, ny, nz, 4, by, bz);
        if (e == cudaSuccess)
            e = encode_map_3d(&tm.u_out, a.u_out, 5ull * a.nx, ny, nz, 5 * kSweepP, by, bz);
        if (e == cudaSuccess && a.w_out)
            e = encode_map_3d(&tm.w_out, a.w_out, 2ull * a.nx, ny, nz, 2 * kSweepP, by, bz);
        if (e != cudaSuccess)
            return e;
        smem = fluidx_sweep_smem_bytes(n);
    }
    k_fluidx2<R, EX, C, T, AX><<<grid, a.P * T, smem, s>>>(a, tm);
    return cudaGetLastError();
}

// Sweep of the untransposed state along y or z (fused step, FP32): pencils
// of n = 4T <= 512 cells along the sweep (one or two tensor boxes), four
// pencils at consecutive x per CTA (nx a multiple of 4, so every box starts
// on a 16-byte boundary), one box of the state.
static bool plan_fluidx_sweep(int n, int nx, int nbox, FxPlan& p)
{
    p = FxPlan{0, 0, 0};
    if (!kV2 || nbox != 1 || n % 4 != 0 || !pow2_in(n / 4, 8, 128) || nx % kSweepP != 0)
        return false;
    p.C = 4, p.T = n / 4, p.P = kSweepP;
    return true;
}

template <int AX>
static cudaError_t fluidx_sweep(FluidxArgs a, const FxPlan& p, cudaStream_t s)
{
    if constexpr (kV2) {
        a.P = p.P;
        switch (p.T) {
        case 8: return launch_fx2<4, 8, AX>(a, s);
        case 16: return launch_fx2<4, 16, AX>(a, s);
        case 32: return launch_fx2<4, 32, AX>(a, s);
        case 64: return launch_fx2<4, 64, AX>(a, s);
        case 128: return launch_fx2<4, 128, AX>(a, s);
        }
    }
    return cudaErrorInvalidValue;
}

// A plane range (kcount) is taken by the x sweep's and the y sweep's
// register-engine kernels (k_fluidx2) of one box, nowhere else.
static bool fluidx_range_ok(const FluidxArgs& a)
{
    if (a.kcount == 0 && a.kbeg == 0)
        return true;
    if (a.kcount <= 0 || a.kbeg < 0 || a.kbeg + a.kcount > a.nz || a.axis == 2 || a.bs.count != 1)
        return false;
    return a.axis == 1 || plan_fluidx(a.nx, a.ny, a.use_tma != 0).C != 0;
}

static cudaError_t fluidx(const FluidxArgs& in, cudaStream_t s)
{
    FluidxArgs a = in;
    if (!fluidx_range_ok(a))
        return cudaErrorInvalidValue;
    if (a.axis != 0) {
        FxPlan p;
        const uintptr_t al = reinterpret_cast<uintptr_t>(a.u_out) | reinterpret_cast<uintptr_t>(a.uu) |
                             reinterpret_cast<uintptr_t>(a.ub);
        if (a.cfl_part || (a.w_out && (a.w_comp < 1 || a.w_comp > 3 || (reinterpret_cast<uintptr_t>(a.w_out) & 15))) ||
            (al & 15) != 0 ||
            !plan_fluidx_sweep(a.axis == 1 ? a.ny : a.nz, a.nx, a.bs.count, p))
            return cudaErrorInvalidValue;
        return (a.axis == 1) ? fluidx_sweep<1>(a, p, s) : fluidx_sweep<2>(a, p, s);
    }
    const FxPlan p = plan_fluidx(a.nx, a.ny, a.use_tma != 0);
    a.P = p.P;
    if constexpr (kV2) {
        if (p.C == 8) {
            switch (p.T) {
            case 8: return launch_fx2<8, 8>(a, s);
            case 16: return launch_fx2<8, 16>(a, s);
            case 32: return launch_fx2<8, 32>(a, s);
            case 64: return launch_fx2<8, 64>(a, s);
            }
        } else if (p.C == 4) {
            switch (p.T) {
            case 8: return launch_fx2<4, 8>(a, s);
            case 16: return launch_fx2<4, 16>(a, s);
            case 32: return launch_fx2<4, 32>(a, s);
            case 64: return launch_fx2<4, 64>(a, s);
            case 128: return launch_fx2<4, 128>(a, s);
            }
        } else if (p.C == 3) {
            switch (p.T) {
            case 16: return launch_fx2<3, 16>(a, s);
            case 32: return launch_fx2<3, 32>(a, s);
            case 64: return launch_fx2<3, 64>(a, s);
            case 128: return launch_fx2<3, 128>(a, s);
            }
        }
    }
    static bool attr = false;
    cudaError_t e = allow_smem(k_fluidx<R, EX>, attr);
    if (e != cudaSuccess)
        return e;
    dim3 grid(a.ny / a.P, a.nz, a.bs.count);
    k_fluidx<R, EX><<<grid, fluidx_threads(a.nx, a.P), fluidx_smem_elems(a.nx, a.P) * sizeof(R), s>>>(a);
    return cudaGetLastError();
}

static int fluidx_parts(int nx, int ny, int nz, int aligned)
{
    const FxPlan p = plan_fluidx(nx, ny, aligned != 0);
    return (ny / p.P) * nz;
}

// -------------------------------------------------------------- advectbyzx

static FxPlan plan_advect(int nx, int ny, bool aligned)
{
    FxPlan p{0, 0, 0};
    if (kV2 && aligned) {
        if (nx % 8 == 0 && pow2_in(nx / 8, 4, 64))
            p.C = 8, p.T = nx / 8;
        else if (nx % 6 == 0 && pow2_in(nx / 6, 8, 64))
            p.C = 6, p.T = nx / 6;
        if (p.C) {
            p.P = 0;
            for (int P = 1; P <= ny && P <= 32; P++)
                if (ny % P == 0 && advect2_threads(P, p.T) <= 512)
                    p.P = P;
            if (p.P)
                return p;
        }
    }
    p.C = p.T = 0;
    p.P = advect_pencils(nx, ny);
    return p;
}

// Marching kernel (FP32): C cells per thread (4 by default, or 8), a ring of
// NS plane slabs (3 by default, or 2), J pencils per CTA (the largest that
// keeps `ctas` CTAs per SM in shared memory) and K planes per CTA (the
// largest that still gives >= 4 waves).  Every choice can be overridden by
// the tuning knobs (advect.cells / slots / J / K).
struct A3Plan {
    int C, T, NS, J, K;
};

static bool plan_advect3(int nx, int ny, int nz, bool aligned, A3Plan& p, int ax = 0, int uc = 5, int boxes = 1)
{
    if (!kV2 || !aligned)
        return false;
    p.C = tune_value(TUNE_ADVECT_C) == 8 ? 8 : 4;
    p.NS = tune_value(TUNE_ADVECT_SLOTS) == 2 ? 2 : 3;  // three slots measured best (autotune.py)
    if (nx % p.C != 0)
        return false;
    p.T = nx / p.C;
    if (!(p.C == 4 ? pow2_in(p.T, 8, 128) : pow2_in(p.T, 4, 64)))
        return false;
    const int ctas = ((p.NS == 2) ? 3 : 2) + (uc < 5 ? 1 : 0);  // the side array leaves room for one more
    const size_t smem_cap = (size_t)(224 * 1024) / ctas;
    const int jt = tune_value(TUNE_ADVECT_J);
    p.J = 0;
    for (int j = 1; j <= ny && j <= 16; j++) {
        const bool fits = advect3_threads(j, p.T) <= 384 && advect3_smem_floats(j, nx, p.NS, ax, uc) * sizeof(float) <= 227 * 1024;
        if (ny % j != 0 || !fits)
            continue;
        if (jt ? (j == jt) : (advect3_smem_floats(j, nx, p.NS, ax, uc) * sizeof(float) <= smem_cap))
            p.J = j;
    }
    if (!p.J)
        return false;
    const int kt = tune_value(TUNE_ADVECT_K);
    p.K = 1;
    for (int k = 1; k <= nz && k <= 64; k++) {
        if (nz % k != 0)
            continue;
        // the launch's CTAs are the boxes' together (a batch class is one launch)
        if (kt ? (k == kt) : ((long long)(ny / p.J) * (nz / k) * boxes >= 4LL * ctas * 152 && k <= 32))
            p.K = k;
    }
    return true;
}

template <int C, int T, int NS, int AX = 0, bool WU = false>
static cudaError_t launch_ad3(const AdvectArgs& a, cudaStream_t s)
{
    static bool attr = false;
    cudaError_t e = allow_smem(k_advect3<EX, C, T, NS, AX, WU>, attr, AX == 0);
    if (e != cudaSuccess)
        return e;
    const int nj = (AX == 0) ? a.ny : a.nx, nk = (AX == 2) ? a.ny : a.nz;
    dim3 grid(nj / a.P, nk / a.K, a.bs.count);
    k_advect3<EX, C, T, NS, AX, WU><<<grid, advect3_threads(a.P, T),
                                      advect3_smem_floats(a.P, C * T, NS, AX, WU ? 2 : 5) * sizeof(float), s>>>(a);
    return cudaGetLastError();
}

template <int C, int NS, int AX = 0, bool WU = false>
static cudaError_t launch_ad3_t(const AdvectArgs& a, int T, cudaStream_t s)
{
    switch (T) {
    case 4: if constexpr (C == 8) return launch_ad3<C, 4, NS, AX, WU>(a, s); break;
    case 8: return launch_ad3<C, 8, NS, AX, WU>(a, s);
    case 16: return launch_ad3<C, 16, NS, AX, WU>(a, s);
    case 32: return launch_ad3<C, 32, NS, AX, WU>(a, s);
    case 64: return launch_ad3<C, 64, NS, AX, WU>(a, s);
    case 128: if constexpr (C == 4) return launch_ad3<C, 128, NS, AX, WU>(a, s); break;
    }
    return cudaErrorInvalidValue;
}

template <int AX>
static cudaError_t advect_sweep(const AdvectArgs& a, const A3Plan& p3, cudaStream_t s)
{
    if (p3.C == 4)
        return (p3.NS == 2) ? launch_ad3_t<4, 2, AX>(a, p3.T, s) : launch_ad3_t<4, 3, AX>(a, p3.T, s);
    return (p3.NS == 2) ? launch_ad3_t<8, 2, AX>(a, p3.T, s) : launch_ad3_t<8, 3, AX>(a, p3.T, s);
}

// x-walking kernel (FP32, the x sweep): the planner's choice for pencils
// longer than 256 cells, where the marching kernel's rows would span more than
// two warps (at 512^3 it measured 1.41 against 3.31 ms per launch), and by the
// knob advect.kernel = 4 otherwise (the marching kernel measured faster at
// 256^3).  KT planes per CTA (4 by default, or advect.xk), NS chunk buffers (2,
// or 3 by advect.slots; 3 when the planner picks the kernel); nx a multiple of
// 4 and ny a multiple of 32.
struct A4Plan {
    int KT, NS;
};

static bool plan_advect4(const AdvectArgs& a, bool aligned, A4Plan& p)
{
    const int kn = tune_value(TUNE_ADVECT_KERNEL);
    const bool long_pencils = (kn == 0 && a.nx > 256);
    if (!kV2 || !aligned || a.axis != 0 || !(kn == 4 || long_pencils))
        return false;
    if (a.nx % kA4X != 0 || a.ny % kA4J != 0)
        return false;
    if ((long long)a.nx * a.ny * a.nz * 5 >= (1LL << 31))  // 32-bit offsets inside a box
        return false;
    const int kt = tune_value(TUNE_ADVECT_XK);
    const int slots = tune_value(TUNE_ADVECT_SLOTS);
    p.NS = (slots == 3 || (long_pencils && slots != 2)) ? 3 : 2;
    p.KT = 0;
    for (int k : {4, 8, 2})
        if (!p.KT && (kt == 0 || kt == k) && a.nz % k == 0)
            p.KT = k;
    return p.KT != 0;
}

// Persistent grid: the CTAs that fit on the device at once, shared among the
// boxes of the launch, each with at least 8 chunks of work.
template <int KT, int NS, bool WU = false>
static cudaError_t launch_ad4(const AdvectArgs& a, cudaStream_t s)
{
    static bool attr = false;
    // occupancy per device (the process may drive several kinds of GPU)
    static int per_sm_of[kMaxOccDevices] = {}, nsm_of[kMaxOccDevices] = {};
    cudaError_t e = allow_smem(k_advect4<EX, KT, NS, WU>, attr, true);
    if (e != cudaSuccess)
        return e;
    const size_t smem = advect4_smem_bytes(KT, NS, WU);
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev < 0 || dev >= kMaxOccDevices)
        return cudaErrorInvalidDevice;
    int& per_sm = per_sm_of[dev];
    int& nsm = nsm_of[dev];
    if (!per_sm) {
        e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_advect4<EX, KT, NS, WU>, advect4_threads(KT),
                                                              smem);
        if (e != cudaSuccess)
            return e;
        if (per_sm < 1)
            return cudaErrorInvalidConfiguration;
    }
    const long long work = (long long)(a.ny / kA4J) * (a.nz / KT) * (a.nx / kA4X);
    long long ctas = ((long long)per_sm * nsm + a.bs.count - 1) / a.bs.count;
    const long long cap = (work / 8 > 0) ? work / 8 : 1;
    if (ctas > cap)
        ctas = cap;
    dim3 grid((unsigned)ctas, 1, a.bs.count);
    k_advect4<EX, KT, NS, WU><<<grid, advect4_threads(KT), smem, s>>>(a);
    return cudaGetLastError();
}

static cudaError_t advect_x4(const AdvectArgs& a, const A4Plan& p, cudaStream_t s)
{
    // the (rho, m_x) side array of the fluidx before, when given, replaces u in the chunks
    const bool wu = a.w != nullptr && (reinterpret_cast<uintptr_t>(a.w) & 15) == 0 &&
                    (a.bs.count == 1 || a.bs.w % 16 == 0);
    if (wu) {
        switch (p.KT * 10 + p.NS) {
        case 82: return launch_ad4<8, 2, true>(a, s);
        case 83: return launch_ad4<8, 3, true>(a, s);
        case 42: return launch_ad4<4, 2, true>(a, s);
        case 43: return launch_ad4<4, 3, true>(a, s);
        case 22: return launch_ad4<2, 2, true>(a, s);
        case 23: return launch_ad4<2, 3, true>(a, s);
        }
        return cudaErrorInvalidValue;
    }
    switch (p.KT * 10 + p.NS) {
    case 82: return launch_ad4<8, 2>(a, s);
    case 83: return launch_ad4<8, 3>(a, s);
    case 42: return launch_ad4<4, 2>(a, s);
    case 43: return launch_ad4<4, 3>(a, s);
    case 22: return launch_ad4<2, 2>(a, s);
    case 23: return launch_ad4<2, 3>(a, s);
    }
    return cudaErrorInvalidValue;
}

// Warp-per-pencil marching kernel (FP32, the x sweep with the side array,
// b(1) read in place; several boxes when their side arrays are contiguous):
// pencils of n = 32 C cells (C = 2, 3, 4, 8), J pencils per CTA (2, or 4 by
// advect.J), K planes per CTA (the largest that gives >= 4 waves, or
// advect.K).  The planner's choice for pencils of 96, 128 and 256 cells (at
// 256^3 it measured 134 against 184 us for the marching kernel), and by
// advect.kernel = 6 for 64.
struct A6Plan {
    int C, J, K;
};

static bool plan_advect6(const AdvectArgs& a, bool aligned, A6Plan& p)
{
    const int kn = tune_value(TUNE_ADVECT_KERNEL);
    if (!kV2 || !aligned || a.axis != 0 || !(kn == 6 || (kn == 0 && (a.nx == 96 || a.nx == 128 || a.nx == 256))))
        return false;
    // several boxes: their side arrays one after the other (one tensor map covers them)
    const bool boxes_ok = a.bs.count == 1 || a.bs.w == (size_t)a.nx * a.ny * a.nz * 8;
    if (a.w == nullptr || (reinterpret_cast<uintptr_t>(a.w) & 15) != 0 || a.b1_src != a.ub || !boxes_ok)
        return false;
    if (a.nx % 32 != 0 || !(a.nx / 32 == 2 || a.nx / 32 == 3 || a.nx / 32 == 4 || a.nx / 32 == 8))
        return false;
    p.C = a.nx / 32;
    const int jt = tune_value(TUNE_ADVECT_J);
    p.J = (jt == 4) ? 4 : 2;  // two pencils per CTA measured best at 256^3 (134 against 150 us)
    if (a.ny % p.J != 0)
        return false;
    const int ctas = advect6_min_ctas(p.J);
    const int kt = tune_value(TUNE_ADVECT_K);
    p.K = 0;
    for (int k = 1; k <= a.nz && k <= 64; k++) {
        if (a.nz % k != 0)
            continue;
        if (kt ? (k == kt) : ((long long)(a.ny / p.J) * (a.nz / k) * a.bs.count >= 4LL * ctas * 152 || k == 1))
            p.K = k;
    }
    return p.K != 0;
}

template <int C, int J>
static cudaError_t launch_ad6(const AdvectArgs& a, int K, cudaStream_t s)
{
    // swizzled side-array rows (one box) for 8 and 4 cells per lane
    constexpr bool SW = (C == 8 || C == 4);
    static bool attr = false;
    cudaError_t e = allow_smem(k_advect6<EX, C, J, SW>, attr, true);
    if (e != cudaSuccess)
        return e;
    AdvectArgs b = a;
    b.P = J;
    b.K = K;
    CUtensorMap wmap{};
    if constexpr (SW) {
        // rows of C cells of every box's side array (contiguous: bs.w is one box's array)
        const uint64_t cells = (uint64_t)a.nx * a.ny * a.nz;
        if (a.bs.count != 1 && a.bs.w != cells * 8)
            return cudaErrorInvalidValue;
        e = encode_map_2d(&wmap, a.w, 2 * C, cells / C * (uint64_t)a.bs.count, 32,
                          C == 8 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
        if (e != cudaSuccess)
            return e;
    }
    dim3 grid(a.ny / J, (a.kcount ? a.kcount : a.nz) / K, a.bs.count);
    k_advect6<EX, C, J, SW><<<grid, advect6_threads(J), advect6_smem_bytes(C * 32, J), s>>>(b, wmap);
    return cudaGetLastError();
}

static cudaError_t advect_x6(const AdvectArgs& a, const A6Plan& p, cudaStream_t s)
{
    switch (p.C * 10 + p.J) {
    case 82: return launch_ad6<8, 2>(a, p.K, s);
    case 84: return launch_ad6<8, 4>(a, p.K, s);
    case 42: return launch_ad6<4, 2>(a, p.K, s);
    case 44: return launch_ad6<4, 4>(a, p.K, s);
    case 32: return launch_ad6<3, 2>(a, p.K, s);
    case 34: return launch_ad6<3, 4>(a, p.K, s);
    case 22: return launch_ad6<2, 2>(a, p.K, s);
    case 24: return launch_ad6<2, 4>(a, p.K, s);
    }
    return cudaErrorInvalidValue;
}

// Sweep-walking kernel of the fused step's sweeps along y and z (FP32, one
// box): lanes along x (nx a multiple of 32), KT planes per CTA (4 by default,
// or sweep.k), NS chunk buffers (3, or 2 by sweep.slots), the pencil length a
// multiple of 4.  sweep.kernel = 3 keeps the marching kernel instead.
static bool plan_advect5(const AdvectArgs& a, A4Plan& p)
{
    if (!kV2 || a.axis == 0 || a.b1_src != a.ub || a.bs.count != 1 || tune_value(TUNE_SWEEP_KERNEL) == 3)
        return false;
    const int n = (a.axis == 1) ? a.ny : a.nz, nk = (a.axis == 1) ? a.nz : a.ny;
    const uintptr_t al = reinterpret_cast<uintptr_t>(a.b_out) | reinterpret_cast<uintptr_t>(a.uu) |
                         reinterpret_cast<uintptr_t>(a.ub);
    if ((al & 15) != 0 || a.nx % kA5J != 0 || n % kA4X != 0)
        return false;
    if ((long long)a.nx * a.ny * a.nz * 5 >= (1LL << 31))  // 32-bit offsets inside the box
        return false;
    const int kt = tune_value(TUNE_SWEEP_K);
    p.NS = (tune_value(TUNE_SWEEP_SLOTS) == 2) ? 2 : 3;
    p.KT = 0;
    for (int k : {4, 8, 2})
        if (!p.KT && (kt == 0 || kt == k) && nk % k == 0)
            p.KT = k;
    return p.KT != 0;
}

template <int KT, int NS, int AX, bool WU = false>
static cudaError_t launch_ad5(const AdvectArgs& a, cudaStream_t s)
{
    static bool attr = false;
    static int per_sm_of[kMaxOccDevices] = {}, nsm_of[kMaxOccDevices] = {};
    cudaError_t e = allow_smem(k_advect5<EX, KT, NS, AX, WU>, attr, true);
    if (e != cudaSuccess)
        return e;
    const size_t smem = advect5_smem_bytes(KT, NS, WU);
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev < 0 || dev >= kMaxOccDevices)
        return cudaErrorInvalidDevice;
    int& per_sm = per_sm_of[dev];
    int& nsm = nsm_of[dev];
    if (!per_sm) {
        e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_advect5<EX, KT, NS, AX, WU>,
                                                              advect5_threads(KT), smem);
        if (e != cudaSuccess)
            return e;
        if (per_sm < 1)
            return cudaErrorInvalidConfiguration;
    }
    const int n = (AX == 1) ? a.ny : a.nz, nk = (AX == 1) ? a.nz : a.ny;
    const long long work = (long long)(a.nx / kA5J) * (nk / KT) * (n / kA4X);
    long long ctas = (long long)per_sm * nsm;
    const long long cap = (work / 8 > 0) ? work / 8 : 1;
    if (ctas > cap)
        ctas = cap;
    k_advect5<EX, KT, NS, AX, WU><<<dim3((unsigned)ctas, 1, 1), advect5_threads(KT), smem, s>>>(a);
    return cudaGetLastError();
}

template <int AX, bool WU>
static cudaError_t advect_y5_w(const AdvectArgs& a, const A4Plan& p, cudaStream_t s)
{
    switch (p.KT * 10 + p.NS) {
    case 82: return launch_ad5<8, 2, AX, WU>(a, s);
    case 83: return launch_ad5<8, 3, AX, WU>(a, s);
    case 42: return launch_ad5<4, 2, AX, WU>(a, s);
    case 43: return launch_ad5<4, 3, AX, WU>(a, s);
    case 22: return launch_ad5<2, 2, AX, WU>(a, s);
    case 23: return launch_ad5<2, 3, AX, WU>(a, s);
    }
    return cudaErrorInvalidValue;
}

// the (rho, m_d) side array of the fluidx before, when given, replaces u in the rows
template <int AX>
static cudaError_t advect_y5(const AdvectArgs& a, const A4Plan& p, cudaStream_t s)
{
    if (a.w != nullptr && (reinterpret_cast<uintptr_t>(a.w) & 15) == 0)
        return advect_y5_w<AX, true>(a, p, s);
    return advect_y5_w<AX, false>(a, p, s);
}

template <int C, int T>
static cudaError_t launch_ad2(const AdvectArgs& a, cudaStream_t s)
{
    static bool attr = false;
    cudaError_t e = allow_smem(k_advect2<R, EX, C, T>, attr);
    if (e != cudaSuccess)
        return e;
    dim3 grid(a.ny / a.P, a.nz, a.bs.count);
    k_advect2<R, EX, C, T><<<grid, advect2_threads(a.P, T), advect2_smem_elems(a.nx, a.P) * sizeof(R), s>>>(a);
    return cudaGetLastError();
}

static cudaError_t advect(const AdvectArgs& in, cudaStream_t s)
{
    AdvectArgs a = in;
    if (a.kcount != 0 || a.kbeg != 0) {  // a plane range: the warp-per-pencil x-sweep kernel only
        const uintptr_t al = reinterpret_cast<uintptr_t>(a.b_out) | reinterpret_cast<uintptr_t>(a.b1_src) |
                             reinterpret_cast<uintptr_t>(a.uu) | reinterpret_cast<uintptr_t>(a.ub);
        A6Plan p6;
        if (a.kcount <= 0 || a.kbeg < 0 || a.kbeg + a.kcount > a.nz || !plan_advect6(a, (al & 15) == 0, p6) ||
            a.kcount % p6.K != 0 || a.kbeg % p6.K != 0)
            return cudaErrorInvalidValue;
        return advect_x6(a, p6, s);
    }
    if (a.axis != 0) {  // fused step: pencils along y or z of the untransposed state
        if constexpr (kV2) {
            A4Plan p5;
            if (plan_advect5(a, p5))
                return (a.axis == 1) ? advect_y5<1>(a, p5, s) : advect_y5<2>(a, p5, s);
        }
        A3Plan p3;
        const int n = (a.axis == 1) ? a.ny : a.nz, nk = (a.axis == 1) ? a.nz : a.ny;
        if (!kV2 || a.b1_src != a.ub || !plan_advect3(n, a.nx, nk, true, p3, a.axis))
            return cudaErrorInvalidValue;
        a.P = p3.J;
        a.K = p3.K;
        return (a.axis == 1) ? advect_sweep<1>(a, p3, s) : advect_sweep<2>(a, p3, s);
    }
    const uintptr_t al = reinterpret_cast<uintptr_t>(a.b_out) | reinterpret_cast<uintptr_t>(a.b1_src) |
                         reinterpret_cast<uintptr_t>(a.uu) | reinterpret_cast<uintptr_t>(a.ub);
    if constexpr (kV2) {
        A6Plan p6;
        if (plan_advect6(a, (al & 15) == 0, p6))
            return advect_x6(a, p6, s);
        A4Plan p4;
        if (plan_advect4(a, (al & 15) == 0, p4))
            return advect_x4(a, p4, s);
        // the (rho, m_x) side array of the fluidx before, when given, replaces u in the slabs
        const bool wu = a.w != nullptr && (reinterpret_cast<uintptr_t>(a.w) & 15) == 0 &&
                        (a.bs.count == 1 || a.bs.w % 16 == 0);
        A3Plan p3;
        if (wu && plan_advect3(a.nx, a.ny, a.nz, (al & 15) == 0, p3, 0, 2, a.bs.count) && p3.C == 4) {
            a.P = p3.J;
            a.K = p3.K;
            return (p3.NS == 2) ? launch_ad3_t<4, 2, 0, true>(a, p3.T, s) : launch_ad3_t<4, 3, 0, true>(a, p3.T, s);
        }
        if (plan_advect3(a.nx, a.ny, a.nz, (al & 15) == 0, p3, 0, 5, a.bs.count)) {
            a.P = p3.J;
            a.K = p3.K;
            if (p3.C == 4)
                return (p3.NS == 2) ? launch_ad3_t<4, 2>(a, p3.T, s) : launch_ad3_t<4, 3>(a, p3.T, s);
            return (p3.NS == 2) ? launch_ad3_t<8, 2>(a, p3.T, s) : launch_ad3_t<8, 3>(a, p3.T, s);
        }
    }
    const FxPlan p = plan_advect(a.nx, a.ny, (al & 15) == 0);
    a.P = p.P;
    if constexpr (kV2) {
        if (p.C == 8) {
            switch (p.T) {
            case 4: return launch_ad2<8, 4>(a, s);
            case 8: return launch_ad2<8, 8>(a, s);
            case 16: return launch_ad2<8, 16>(a, s);
            case 32: return launch_ad2<8, 32>(a, s);
            case 64: return launch_ad2<8, 64>(a, s);
            }
        } else if (p.C == 6) {
            switch (p.T) {
            case 8: return launch_ad2<6, 8>(a, s);
            case 16: return launch_ad2<6, 16>(a, s);
            case 32: return launch_ad2<6, 32>(a, s);
            case 64: return launch_ad2<6, 64>(a, s);
            }
        }
    }
    static bool attr = false;
    cudaError_t e = allow_smem(k_advect<R, EX>, attr);
    if (e != cudaSuccess)
        return e;
    int threads = ((a.nx * a.P + 31) / 32) * 32;
    if (threads > 512)
        threads = 512;
    if (threads < 128)
        threads = 128;
    dim3 grid(a.ny / a.P, a.nz, a.bs.count);
    k_advect<R, EX><<<grid, threads, advect_smem_elems(a.nx, a.P) * sizeof(R), s>>>(a);
    return cudaGetLastError();
}

// -------------------------------------------------------------- transposes

static cudaError_t transpose(const TransposeArgs& a, cudaStream_t s)
{
    const int na = (a.axis == 1) ? a.ny : a.nz;
    const int nb = (a.axis == 1) ? a.nz : a.ny;
    if constexpr (kV2) {
        const uintptr_t al = reinterpret_cast<uintptr_t>(a.u_out) | reinterpret_cast<uintptr_t>(a.b_out) |
                             reinterpret_cast<uintptr_t>(a.uu) | reinterpret_cast<uintptr_t>(a.ub);
        if (a.nx % kT3 == 0 && na % kT3 == 0 && (al & 15) == 0) {  // bulk-TMA tiles
            dim3 grid(a.nx / kT3, na / kT3, nb * a.bs.count);
            if (a.axis == 1)
                k_transpose3<1><<<grid, 256, 0, s>>>(a);
            else
                k_transpose3<2><<<grid, 256, 0, s>>>(a);
            return cudaGetLastError();
        }
        if (a.nx % 16 == 0 && na % 16 == 0 && (al & 15) == 0) {  // bulk-TMA tiles of 16 cells
            dim3 grid(a.nx / 16, na / 16, nb * a.bs.count);
            if (a.axis == 1)
                k_transpose3<1, 16><<<grid, 256, 0, s>>>(a);
            else
                k_transpose3<2, 16><<<grid, 256, 0, s>>>(a);
            return cudaGetLastError();
        }
        if (a.nx % kT2 == 0 && na % kT2 == 0 && (al & 3) == 0) {
            dim3 grid(a.nx / kT2, na / kT2, nb * a.bs.count);
            if (a.axis == 1)
                k_transpose2<1><<<grid, 256, 0, s>>>(a);
            else
                k_transpose2<2><<<grid, 256, 0, s>>>(a);
            return cudaGetLastError();
        }
    }
    constexpr int T = TTile<R>::E;
    dim3 grid((a.nx + T - 1) / T, (na + T - 1) / T, nb * a.bs.count);
    k_transpose<R><<<grid, 256, 0, s>>>(a);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ calcfl

static cudaError_t calcfl(const void* u, const void* b, size_t ncell, size_t cell0, void* part, int* nparts,
                          const BoxStrides& bs, cudaStream_t s)
{
    const int blocks = (int)((ncell + 255) / 256);
    *nparts = blocks;
    k_calcfl<R, EX><<<dim3(blocks, bs.count), 256, 0, s>>>(static_cast<const R*>(u), static_cast<const R*>(b), ncell,
                                                           cell0, static_cast<CflPart<R>*>(part), bs);
    return cudaGetLastError();
}

static cudaError_t cfl_finalize(const CflFinalizeArgs& in, cudaStream_t s)
{
    CflFinalizeArgs a = in;
    if (a.bs.count == 1 && a.scratch && a.nparts > kCflReduceMin) {
        int g = (a.nparts + 511) / 512;
        g = g < kCflReduceCtas ? g : kCflReduceCtas;
        k_cfl_reduce<R><<<g, 256, 0, s>>>(static_cast<const CflPart<R>*>(a.part), a.nparts,
                                          static_cast<CflPart<R>*>(a.scratch));
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
            return e;
        a.part = a.scratch;
        a.nparts = g;
    }
    k_cfl_finalize<R, EX><<<a.bs.count, 1024, 0, s>>>(a);
    return cudaGetLastError();
}

static cudaError_t divb(const void* b, int nx, int ny, int nz, double* part, int* nparts, cudaStream_t s)
{
    const size_t ncell = (size_t)nx * ny * nz;
    const int blocks = (int)((ncell + 255) / 256);
    *nparts = blocks;
    k_divb<R><<<blocks, 256, 0, s>>>(static_cast<const R*>(b), nx, ny, nz, part);
    return cudaGetLastError();
}

// the fused step's sweeps along y and z have kernels for this shape (one box)
static int fused_ok(int nx, int ny, int nz)
{
    FxPlan p;
    A3Plan q;
    A4Plan q5;
    auto advect_ok = [&](int axis) {
        AdvectArgs a{};
        a.nx = nx, a.ny = ny, a.nz = nz, a.axis = axis, a.bs.count = 1;
        const int n = (axis == 1) ? ny : nz, nk = (axis == 1) ? nz : ny;
        return plan_advect5(a, q5) || plan_advect3(n, nx, nk, true, q, axis);
    };
    return plan_fluidx_sweep(ny, nx, 1, p) && plan_fluidx_sweep(nz, nx, 1, p) && advect_ok(1) && advect_ok(2);
}

// nonzero if the x-sweep fluidx of this grid is k_fluidx2 (which writes the
// (rho, m_x) side array when asked)
static int fluidx_writes_w(int nx, int ny, int nz, int aligned)
{
    (void)nz;
    return kV2 && plan_fluidx(nx, ny, aligned != 0).C != 0;
}

// nonzero if the transpose of this grid is k_transpose3 (which writes the side
// array when asked); nx, ny, nz are the input dims, the buffers 16-byte aligned
static int transpose_writes_w(int axis, int nx, int ny, int nz)
{
    const int na = (axis == 1) ? ny : nz;
    return kV2 && nx % kT3 == 0 && na % kT3 == 0;
}

// nonzero if the fused step's fluidx sweep along `axis` (1: y, 2: z) of this
// grid writes the side array when asked
static int sweep_writes_w(int axis, int nx, int ny, int nz)
{
    FxPlan p;
    return kV2 && (axis == 1 || axis == 2) && plan_fluidx_sweep(axis == 1 ? ny : nz, nx, 1, p);
}

static int tail_slabs_ok(int nx, int ny, int nz, int kcount)
{
    if (!kV2 || kcount <= 0 || nz % kcount != 0 || !sweep_writes_w(1, nx, ny, nz))
        return 0;
    FxPlan p;
    const bool aligned = ((size_t)nx * 5 * sizeof(R)) % 16 == 0 && ((size_t)nx * 3 * sizeof(R)) % 16 == 0;
    if (!plan_fluidx_sweep(ny, nx, 1, p) || plan_fluidx(nx, ny, aligned).C == 0)
        return 0;
    // the x-sweep advectbyzx with a side array (any 16-byte aligned address stands in for the buffers)
    AdvectArgs a{};
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    a.ub = a.b1_src = a.w = reinterpret_cast<const void*>(uintptr_t(256));
    A6Plan p6;
    return (plan_advect6(a, aligned, p6) && kcount % p6.K == 0) ? 1 : 0;
}

static int batch_side_ok(int n, int boxes)
{
    const bool aligned = ((size_t)n * 5 * sizeof(R)) % 16 == 0 && ((size_t)n * 3 * sizeof(R)) % 16 == 0;
    if (!kV2 || boxes < 1 || plan_fluidx(n, n, aligned).C == 0)  // the x-sweep fluidx writes it
        return 0;
    AdvectArgs a{};  // any 16-byte aligned address stands in for the buffers
    a.nx = a.ny = a.nz = n;
    a.ub = a.b1_src = a.w = reinterpret_cast<const void*>(uintptr_t(256));
    a.bs.count = boxes;
    a.bs.w = (size_t)n * n * n * 8;
    A6Plan p6;
    return plan_advect6(a, aligned, p6) ? 1 : 0;
}

// --------------------------------------------- work-list launches (batch)
//
// One launch per operator over several size classes of cubes (mhd_multi.cuh):
// `in` holds one argument set per class (nx = ny = nz = n, the class's box
// strides and count), in launch order.  FP32 only; the classes' edges must be
// those multi_ok accepts, their buffers 16-byte aligned, and the advectbyzx
// arguments must carry the class's side array (contiguous over its boxes).

static int multi_ok(int n) { return (kV2 && multi_kind_of_edge(n) >= 0) ? 1 : 0; }

// CFL partials per box written by the work-list fluidx (one per CTA)
static int multi_fluidx_parts(int n)
{
    const int T = multi_fx_threads(n);
    return T ? (n / (kMultiFxThreads / T)) * n : 0;
}

// the advectbyzx CTA's planes along k for a class of `count` boxes of edge n
// (the rule of plan_advect6: the largest K <= 64 that still gives 4 waves)
static int multi_advect_k(int n, int count)
{
    const int ctas = advect6_min_ctas(kMultiAdJ);
    int K = 1;
    for (int k = 1; k <= n && k <= 64; k++)
        if (n % k == 0 && (long long)(n / kMultiAdJ) * (n / k) * count >= 4LL * ctas * 152)
            K = k;
    return K;
}

static bool multi_args_ok(int nseg, const int* edges)
{
    if (!kV2 || nseg < 1 || nseg > kMaxSegs)
        return false;
    for (int i = 0; i < nseg; i++)
        if (!multi_ok(edges[i]))
            return false;
    return true;
}

static cudaError_t fluidx_multi(const FluidxArgs* in, int nseg, cudaStream_t s)
{
    if constexpr (kV2) {
        int edges[kMaxSegs];
        for (int i = 0; i < nseg && i < kMaxSegs; i++)
            edges[i] = in[i].nx;
        if (!multi_args_ok(nseg, edges))
            return cudaErrorInvalidValue;
        static bool attr = false;
        cudaError_t e = allow_smem(k_fluidx2_multi<R, EX>, attr, true);
        if (e != cudaSuccess)
            return e;
        FluidxMulti m{};
        long long total = 0;
        size_t smem = 0;
        for (int i = 0; i < nseg; i++) {
            const int n = in[i].nx, T = multi_fx_threads(n), P = kMultiFxThreads / T;
            m.a[i] = in[i];
            m.a[i].P = P;
            m.a[i].use_tma = 1;
            m.g[i] = SegGrid{(int)total, n / P, n, multi_kind_of_edge(n)};
            total += (long long)(n / P) * n * in[i].bs.count;
            const size_t sm = fluidx2_smem_elems(n, P) * sizeof(R);
            smem = sm > smem ? sm : smem;
        }
        m.nseg = nseg;
        if (total <= 0 || total >= (1LL << 31))
            return cudaErrorInvalidValue;
        k_fluidx2_multi<R, EX><<<(unsigned)total, kMultiFxThreads, smem, s>>>(m);
        return cudaGetLastError();
    } else {
        (void)in, (void)nseg, (void)s;
        return cudaErrorNotSupported;
    }
}

static cudaError_t advect_multi(const AdvectArgs* in, int nseg, cudaStream_t s)
{
    if constexpr (kV2) {
        int edges[kMaxSegs];
        for (int i = 0; i < nseg && i < kMaxSegs; i++)
            edges[i] = in[i].nx;
        if (!multi_args_ok(nseg, edges))
            return cudaErrorInvalidValue;
        static bool attr = false;
        cudaError_t e = allow_smem(k_advect6_multi<EX>, attr, true);
        if (e != cudaSuccess)
            return e;
        AdvectMulti m{};
        long long total = 0;
        size_t smem = 0;
        for (int i = 0; i < nseg; i++) {
            const AdvectArgs& a = in[i];
            const int n = a.nx, kind = multi_kind_of_edge(n);
            const uint64_t cells = (uint64_t)n * n * n;
            const uintptr_t al = reinterpret_cast<uintptr_t>(a.b_out) | reinterpret_cast<uintptr_t>(a.b1_src) |
                                 reinterpret_cast<uintptr_t>(a.uu) | reinterpret_cast<uintptr_t>(a.ub) |
                                 reinterpret_cast<uintptr_t>(a.w);
            if (!a.w || (al & 15) != 0 || a.b1_src != a.ub || a.axis != 0 || a.kcount != 0 || a.kbeg != 0 ||
                (a.bs.count != 1 && a.bs.w != cells * 8))
                return cudaErrorInvalidValue;
            const int K = multi_advect_k(n, a.bs.count);
            m.a[i] = a;
            m.a[i].P = kMultiAdJ;
            m.a[i].K = K;
            if (kind == MAD_4_32) {  // 4 cells per lane: swizzled side-array rows, one map over the boxes
                e = encode_map_2d(&m.wmap[i], a.w, 8, cells / 4 * (uint64_t)a.bs.count, 32,
                                  CU_TENSOR_MAP_SWIZZLE_32B);
                if (e != cudaSuccess)
                    return e;
            }
            m.g[i] = SegGrid{(int)total, n / kMultiAdJ, n / K, kind};
            total += (long long)(n / kMultiAdJ) * (n / K) * a.bs.count;
            const size_t sm = advect6_smem_bytes(n, kMultiAdJ);
            smem = sm > smem ? sm : smem;
        }
        m.nseg = nseg;
        if (total <= 0 || total >= (1LL << 31))
            return cudaErrorInvalidValue;
        k_advect6_multi<EX><<<(unsigned)total, advect6_threads(kMultiAdJ), smem, s>>>(m);
        return cudaGetLastError();
    } else {
        (void)in, (void)nseg, (void)s;
        return cudaErrorNotSupported;
    }
}

static cudaError_t transpose_multi(const TransposeArgs* in, int nseg, cudaStream_t s)
{
    if constexpr (kV2) {
        int edges[kMaxSegs];
        for (int i = 0; i < nseg && i < kMaxSegs; i++)
            edges[i] = in[i].nx;
        if (!multi_args_ok(nseg, edges))
            return cudaErrorInvalidValue;
        const int axis = in[0].axis;
        TransposeMulti m{};
        long long total = 0;
        for (int i = 0; i < nseg; i++) {
            const TransposeArgs& a = in[i];
            const uintptr_t al = reinterpret_cast<uintptr_t>(a.u_out) | reinterpret_cast<uintptr_t>(a.b_out) |
                                 reinterpret_cast<uintptr_t>(a.uu) | reinterpret_cast<uintptr_t>(a.ub) |
                                 reinterpret_cast<uintptr_t>(a.w_out);
            if (a.axis != axis || (axis != 1 && axis != 2) || (al & 15) != 0)
                return cudaErrorInvalidValue;
            const int n = a.nx;
            const int kind = (n % 32 == 0) ? 0 : ((n % 16 == 0) ? 2 : 1);
            const int E = (kind == 0) ? 32 : ((kind == 2) ? 16 : TTile<float>::E);
            const int g = (n + E - 1) / E;
            m.a[i] = a;
            m.g[i] = SegGrid{(int)total, g, g, kind};
            total += (long long)g * g * n * a.bs.count;
        }
        m.nseg = nseg;
        if (total <= 0 || total >= (1LL << 31))
            return cudaErrorInvalidValue;
        if (axis == 1)
            k_transpose_multi<1><<<(unsigned)total, 256, kMultiTransposeSmem, s>>>(m);
        else
            k_transpose_multi<2><<<(unsigned)total, 256, kMultiTransposeSmem, s>>>(m);
        return cudaGetLastError();
    } else {
        (void)in, (void)nseg, (void)s;
        return cudaErrorNotSupported;
    }
}

static cudaError_t finalize_multi(const CflFinalizeArgs* in, int nseg, cudaStream_t s)
{
    if (nseg < 1 || nseg > kMaxSegs)
        return cudaErrorInvalidValue;
    FinalizeMulti m{};
    long long total = 0;
    for (int i = 0; i < nseg; i++) {
        m.a[i] = in[i];
        m.a[i].scratch = nullptr;
        if (i > 0)
            m.a[i].nsteps = nullptr;  // counted once per launch (box 0 of the first class)
        m.g[i] = SegGrid{(int)total, in[i].bs.count, 1, 0};
        total += in[i].bs.count;
    }
    m.nseg = nseg;
    k_cfl_finalize_multi<R, EX><<<(unsigned)total, 1024, 0, s>>>(m);
    return cudaGetLastError();
}

static const KernelSet kSet = {(int)sizeof(R), EX ? 1 : 0, fluidx, advect, transpose, calcfl, cfl_finalize, divb,
                               sizeof(CflPart<R>), fluidx_parts, fused_ok, fluidx_writes_w, transpose_writes_w,
                               sweep_writes_w, tail_slabs_ok, batch_side_ok, multi_ok, multi_fluidx_parts,
                               fluidx_multi, advect_multi, transpose_multi, finalize_multi};

}  // namespace MHD_SET_NAME
}  // namespace mhd
