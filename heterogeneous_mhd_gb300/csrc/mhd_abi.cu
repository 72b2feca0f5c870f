// C ABI of mhd_gb300 (include/mhd_gb300.h): the drop-in functions with the
// reference's names (C/spu_function.h:1-15), the context API, the Strang step
// driver (C/mhd.c:59-124) and its CUDA-graph capture.  Host code only; every
// computation runs in the kernels of mhd_kernels.cuh.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/mhd_gb300.h"
#include "../../include/mhd_cuda_compat.h"
#include "mhd_launch.h"

using namespace mhd;

// ----------------------------------------------------------------- status

static thread_local int g_last_error = MHD_OK;

static int set_err(int e)
{
    g_last_error = e;
    return e;
}

#define CUDA_TRY(call)                                                                    \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            if (getenv("MHD_GB300_DEBUG"))                                                \
                fprintf(stderr, "mhd_gb300: %s failed: %s (%s:%d)\n", #call,              \
                        cudaGetErrorString(e_), __FILE__, __LINE__);                      \
            return (e_ == cudaErrorMemoryAllocation) ? MHD_ERR_NOMEM : MHD_ERR_CUDA;     \
        }                                                                                 \
    } while (0)

#define MHD_TRY(call)                  \
    do {                               \
        int s_ = (call);               \
        if (s_ != MHD_OK)              \
            return s_;                 \
    } while (0)

extern "C" MHD_API int mhd_last_error(void) { return g_last_error; }

extern "C" MHD_API const char* mhd_error_string(int status)
{
    switch (status) {
    case MHD_OK: return "ok";
    case MHD_ERR_ARG: return "bad argument";
    case MHD_ERR_CUDA: return "CUDA runtime error";
    case MHD_ERR_TIMEOUT: return "device-side wait timed out";
    case MHD_ERR_NONFINITE: return "non-finite value in the CFL reduction";
    case MHD_ERR_UNSUPPORTED: return "unsupported shape or mode";
    case MHD_ERR_NOMEM: return "device allocation failed";
    default: return "unknown status";
    }
}

// ---------------------------------------------------------------- context

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes)
    {
        if (bytes <= cap)
            return MHD_OK;
        if (p)
            cudaFree(p);
        p = nullptr;
        cap = 0;
        if (bytes == 0)
            return MHD_OK;
        CUDA_TRY(cudaMalloc(&p, bytes));
        cap = bytes;
        return MHD_OK;
    }
    void release()
    {
        if (p)
            cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

struct Pending {
    int kernel;
    cudaEvent_t a, b;
};

struct mhd_ctx {
    int nx, ny, nz, flags;
    const KernelSet* ks;
    int elem;
    int device;
    cudaStream_t stream = nullptr;
    DevBuf U[2], B[2];  // ping-pong state; the current state is (U[0], B[0])
    DevBuf part;        // CFL partials of the step (the last fluidx's epilogue or ensure_cfl)
    DevBuf clock;       // R[4]: t, tf, dt, 1/c
    DevBuf opart;       // partials of the standalone calcfl (mhd_op_calcfl, drop-in calcfl): never the
                        // step's, so a standalone call neither changes the next step's dt nor
                        // reallocates a buffer that a captured step graph reads
    DevBuf opclock;     // result slot of the standalone calcfl (R[4]; only 1/c is written)
    DevBuf misc;        // err (int) + nsteps (long long) + divb partial scratch
    DevBuf stage[4];    // drop-in host staging
    DevBuf alias[2];    // private copies of inputs that alias an output
    DevBuf divb;
    DevBuf cflred;      // first-level CFL reduction results (kCflReduceCtas partials)
    DevBuf W;           // (rho, m_x) side array of the plain step (FP32): forward fluidx and backward
                        // transposes write it, every advectbyzx reads it
    int* err_dev = nullptr;
    long long* nsteps_dev = nullptr;
    // host-buffer steps (mhd_step_host): the copy stream, its events, and the
    // host arrays the last step's result goes to (set only while that step is
    // enqueued; the step copies b out after its last advectbyzx, u after its
    // last fluidx)
    cudaStream_t cstream = nullptr;
    std::vector<cudaEvent_t> cev;
    void* out_u = nullptr;
    void* out_b = nullptr;
    int slab_beg = 0, slab_count = 0;  // plane range along z of the next operators (0 planes: all)
    bool have_state = false;
    bool cfl_valid = false;  // part holds the CFL partials of the current state
    int cfl_nparts = 0;
    // graphs, one per step variant
    int use_graphs = 1;
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    double gcfl[2] = {0, 0};
    long long gtune[2] = {-1, -1};  // tuning generation each graph was captured with
    int glaunches[2] = {0, 0};
    bool capturing = false;
    // profiling
    int profile = 0;
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> ev_free;
    double total_ms[MHD_K_COUNT] = {0};
    long long nlaunch[MHD_K_COUNT] = {0};
    long long launch_count = 0;
};

static size_t ncell(const mhd_ctx* c) { return (size_t)c->nx * c->ny * c->nz; }

// Bulk-TMA rules for x-pencils of the context's element type (the state
// buffers come from cudaMalloc and are 256-byte aligned).
static int tma_ok(const mhd_ctx* c, int nx)
{
    return ((size_t)nx * 5 * c->elem) % 16 == 0 && ((size_t)nx * 3 * c->elem) % 16 == 0;
}

// CFL partials written by the epilogue of the step's last fluidx.
static size_t fluidx_parts(const mhd_ctx* c)
{
    return (size_t)c->ks->fluidx_parts(c->nx, c->ny, c->nz, tma_ok(c, c->nx));
}

static cudaEvent_t ev_get(mhd_ctx* c)
{
    if (!c->ev_free.empty()) {
        cudaEvent_t e = c->ev_free.back();
        c->ev_free.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Brackets one kernel launch with events when profiling (never while capturing).
struct KTimer {
    mhd_ctx* c;
    int id;
    cudaEvent_t a = nullptr, b = nullptr;
    KTimer(mhd_ctx* ctx, int kid) : c(ctx), id(kid)
    {
        c->launch_count++;
        if (c->profile && !c->capturing) {
            a = ev_get(c);
            b = ev_get(c);
            cudaEventRecord(a, c->stream);
        }
    }
    ~KTimer()
    {
        if (a) {
            cudaEventRecord(b, c->stream);
            c->pending.push_back({id, a, b});
        }
    }
};

static void drain_profile(mhd_ctx* c)
{
    if (c->pending.empty())
        return;
    cudaStreamSynchronize(c->stream);
    for (auto& p : c->pending) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            c->total_ms[p.kernel] += ms;
            c->nlaunch[p.kernel] += 1;
        }
        c->ev_free.push_back(p.a);
        c->ev_free.push_back(p.b);
    }
    c->pending.clear();
}

static const KernelSet* pick_set(int flags)
{
    const bool f64 = (flags & MHD_F64) != 0;
    const bool ex = (flags & MHD_MODE_EXACT) != 0;
    if (f64)
        return kernels_f64_exact();  // the FP64 build follows the reference's order
    return ex ? kernels_f32_exact() : kernels_f32_fast();
}

static int check_dims(int nx, int ny, int nz)
{
    if (nx <= 0 || ny <= 0 || nz <= 0)
        return MHD_ERR_ARG;
    if (nx > 512 || ny > 65535 * 64 || nz > 65535)
        return MHD_ERR_UNSUPPORTED;
    return MHD_OK;
}

static void invalidate_graphs(mhd_ctx* c)
{
    for (int v = 0; v < 2; v++)
        if (c->gexec[v]) {
            cudaGraphExecDestroy(c->gexec[v]);
            c->gexec[v] = nullptr;
        }
}

extern "C" MHD_API int mhd_create(mhd_ctx** out, int nx, int ny, int nz, int flags)
{
    if (!out || nx <= 0 || ny <= 0 || nz <= 0)
        return set_err(MHD_ERR_ARG);
    *out = nullptr;
    mhd_ctx* c = new mhd_ctx();
    c->nx = nx;
    c->ny = ny;
    c->nz = nz;
    c->flags = flags;
    c->ks = pick_set(flags);
    c->elem = c->ks->elem;
    if (cudaGetDevice(&c->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return set_err(MHD_ERR_CUDA);
    }
    int s = c->clock.ensure(4 * sizeof(double));
    if (s == MHD_OK)
        s = c->misc.ensure(64);
    if (s != MHD_OK) {
        cudaStreamDestroy(c->stream);
        delete c;
        return set_err(s);
    }
    c->err_dev = static_cast<int*>(c->misc.p);
    c->nsteps_dev = reinterpret_cast<long long*>(static_cast<char*>(c->misc.p) + 8);
    cudaMemsetAsync(c->misc.p, 0, 64, c->stream);
    // clock: t = 0, tf = +inf
    if (c->elem == 4) {
        float h[4] = {0.f, INFINITY, 0.f, 0.f};
        cudaMemcpyAsync(c->clock.p, h, sizeof(h), cudaMemcpyHostToDevice, c->stream);
    } else {
        double h[4] = {0.0, INFINITY, 0.0, 0.0};
        cudaMemcpyAsync(c->clock.p, h, sizeof(h), cudaMemcpyHostToDevice, c->stream);
    }
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
        cudaStreamDestroy(c->stream);
        delete c;
        return set_err(MHD_ERR_CUDA);
    }
    *out = c;
    return set_err(MHD_OK);
}

extern "C" MHD_API int mhd_destroy(mhd_ctx* c)
{
    if (!c)
        return MHD_ERR_ARG;
    cudaStreamSynchronize(c->stream);
    drain_profile(c);
    invalidate_graphs(c);
    for (auto& e : c->ev_free)
        cudaEventDestroy(e);
    if (c->cstream) {
        cudaStreamSynchronize(c->cstream);
        cudaStreamDestroy(c->cstream);
    }
    for (auto& e : c->cev)
        cudaEventDestroy(e);
    for (int v = 0; v < 2; v++) {
        c->U[v].release();
        c->B[v].release();
    }
    c->part.release();
    c->clock.release();
    c->opart.release();
    c->opclock.release();
    c->cflred.release();
    c->W.release();
    c->misc.release();
    c->divb.release();
    for (auto& s : c->stage)
        s.release();
    for (auto& s : c->alias)
        s.release();
    cudaStreamDestroy(c->stream);
    delete c;
    return MHD_OK;
}

extern "C" MHD_API void* mhd_stream(mhd_ctx* c) { return c ? (void*)c->stream : nullptr; }

extern "C" MHD_API int mhd_sync(mhd_ctx* c)
{
    if (!c)
        return MHD_ERR_ARG;
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return MHD_OK;
}

// ------------------------------------------------------------ operators

static int op_fluidx(mhd_ctx* c, void* u, const void* uu, const void* ub, int nx, int ny, int nz, double dt,
                     const void* dt_dev, void* cfl_part, int axis = 0, void* w_out = nullptr, int w_comp = 1)
{
    MHD_TRY(check_dims(nx, ny, nz));
    FluidxArgs a{};
    a.u_out = u;
    a.uu = uu;
    a.ub = ub;
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    a.P = fluidx_pencils(nx, ny);
    const uintptr_t al = reinterpret_cast<uintptr_t>(u) | reinterpret_cast<uintptr_t>(uu) |
                         reinterpret_cast<uintptr_t>(ub);
    a.use_tma = ((al & 15) == 0) && ((size_t)nx * 5 * c->elem) % 16 == 0 && ((size_t)nx * 3 * c->elem) % 16 == 0;
    a.dt_val = dt;
    a.dt_ptr = dt_dev;
    a.cfl_part = cfl_part;
    a.err = c->err_dev;
    a.axis = axis;
    a.w_out = w_out;
    a.w_comp = w_comp;
    a.kbeg = c->slab_beg;
    a.kcount = c->slab_count;
    KTimer kt(c, MHD_K_FLUIDX);
    CUDA_TRY(c->ks->fluidx(a, c->stream));
    return MHD_OK;
}

static int op_advect(mhd_ctx* c, void* b_out, const void* b1_src, const void* uu, const void* ub, int nx, int ny,
                     int nz, double dt, const void* dt_dev, int axis = 0, const void* w = nullptr)
{
    MHD_TRY(check_dims(nx, ny, nz));
    AdvectArgs a{};
    a.b_out = b_out;
    a.b1_src = b1_src;
    a.uu = uu;
    a.ub = ub;
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    a.P = advect_pencils(nx, ny);
    a.dt_val = dt;
    a.dt_ptr = dt_dev;
    a.err = c->err_dev;
    a.axis = axis;
    a.w = w;
    a.kbeg = c->slab_beg;
    a.kcount = c->slab_count;
    KTimer kt(c, MHD_K_ADVECT);
    CUDA_TRY(c->ks->advect(a, c->stream));
    return MHD_OK;
}

// transpose13 takes nx == nz (C/transpose13.c:50-61); `degenerate` also lets
// nz == 1 or nx == 1 through, the two extra cases of the reference's CUDA
// wrapper (Cuda/cuda_transpose13.cu:27-42), which the general kernel covers.
static int op_transpose(mhd_ctx* c, int axis, void* u, void* b, const void* uu, const void* ub, int nx, int ny,
                        int nz, void* w_out = nullptr, bool degenerate = false)
{
    if (nx <= 0 || ny <= 0 || nz <= 0)
        return MHD_ERR_ARG;
    if (axis == 2 && nx != nz && !(degenerate && (nx == 1 || nz == 1)))
        return MHD_ERR_ARG;
    TransposeArgs a{u, b, uu, ub, nx, ny, nz, axis};
    a.err = c->err_dev;
    a.w_out = w_out;
    KTimer kt(c, axis == 1 ? MHD_K_TRANSPOSE12 : MHD_K_TRANSPOSE13);
    CUDA_TRY(c->ks->transpose(a, c->stream));
    return MHD_OK;
}

static int op_copy(mhd_ctx* c, const void* src, void* dst, size_t bytes)
{
    if (src == dst || bytes == 0)
        return MHD_OK;
    KTimer kt(c, MHD_K_COPY);
    CUDA_TRY(launch_copy(src, dst, bytes, c->stream));
    return MHD_OK;
}

// First CFL pass into `dst` (grown to fit); returns the partial count in *np.
static int op_calcfl_partials(mhd_ctx* c, DevBuf& dst, const void* u, const void* b, size_t cells, int* np)
{
    MHD_TRY(dst.ensure(((cells + 255) / 256 + 1) * c->ks->part_bytes));
    KTimer kt(c, MHD_K_CALCFL);
    CUDA_TRY(c->ks->calcfl(u, b, cells, 0, dst.p, np, BoxStrides{}, c->stream));
    return MHD_OK;
}

// Reduces `nparts` partials of `part` into the clock `clock` (advance: the
// step's dt, clamp and t += 2 dt; otherwise only 1/c).
static int op_finalize(mhd_ctx* c, const void* part, void* clock, int nparts, const void* u, const void* b, int nx,
                       int ny, int nz, double cfl, int advance)
{
    CflFinalizeArgs a{};
    a.part = part;
    a.nparts = nparts;
    a.u = u;
    a.b = b;
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    a.cfl = cfl;
    a.advance = advance;
    a.clock = clock;
    a.nsteps = c->nsteps_dev;
    a.err = c->err_dev;
    a.scratch = c->cflred.p;
    KTimer kt(c, MHD_K_FINALIZE);
    if (a.scratch && nparts > kCflReduceMin)
        c->launch_count++;  // the first-level reduction kernel
    CUDA_TRY(c->ks->cfl_finalize(a, c->stream));
    return MHD_OK;
}

extern "C" MHD_API int mhd_op_fluidx(mhd_ctx* c, void* u, const void* uu, const void* ub, int nx, int ny, int nz,
                                     double dt)
{
    if (!c || !u || !uu || !ub)
        return set_err(MHD_ERR_ARG);
    return set_err(op_fluidx(c, u, uu, ub, nx, ny, nz, dt, nullptr, nullptr));
}

extern "C" MHD_API int mhd_op_advectbyzx(mhd_ctx* c, void* b, const void* uu, const void* ub, int nx, int ny,
                                         int nz, double dt)
{
    if (!c || !b || !uu || !ub)
        return set_err(MHD_ERR_ARG);
    const void* src = ub;
    if (b == ub) {  // the fused kernel reads neighbour rows of update_b: keep a private copy
        const size_t bytes = (size_t)nx * ny * nz * 3 * c->elem;
        MHD_TRY(set_err(c->alias[1].ensure(bytes)));
        MHD_TRY(set_err(op_copy(c, ub, c->alias[1].p, bytes)));
        src = c->alias[1].p;
    }
    return set_err(op_advect(c, b, b, uu, src, nx, ny, nz, dt, nullptr));
}

static int transpose_entry(mhd_ctx* c, int axis, void* u, void* b, const void* uu, const void* ub, int nx, int ny,
                           int nz)
{
    if (!c || !u || !b || !uu || !ub)
        return MHD_ERR_ARG;
    if (axis == 2 && nx != nz)
        return MHD_ERR_ARG;
    const size_t cells = (size_t)nx * ny * nz;
    if (u == uu) {
        MHD_TRY(c->alias[0].ensure(cells * 5 * c->elem));
        MHD_TRY(op_copy(c, uu, c->alias[0].p, cells * 5 * c->elem));
        uu = c->alias[0].p;
    }
    if (b == ub) {
        MHD_TRY(c->alias[1].ensure(cells * 3 * c->elem));
        MHD_TRY(op_copy(c, ub, c->alias[1].p, cells * 3 * c->elem));
        ub = c->alias[1].p;
    }
    return op_transpose(c, axis, u, b, uu, ub, nx, ny, nz);
}

extern "C" MHD_API int mhd_op_transpose12(mhd_ctx* c, void* u, void* b, const void* uu, const void* ub, int nx,
                                          int ny, int nz)
{
    return set_err(transpose_entry(c, 1, u, b, uu, ub, nx, ny, nz));
}

extern "C" MHD_API int mhd_op_transpose13(mhd_ctx* c, void* u, void* b, const void* uu, const void* ub, int nx,
                                          int ny, int nz)
{
    return set_err(transpose_entry(c, 2, u, b, uu, ub, nx, ny, nz));
}

extern "C" MHD_API int mhd_op_copy(mhd_ctx* c, const void* u, const void* b, void* uu, void* ub, int nx, int ny,
                                   int nz)
{
    if (!c || !u || !b || !uu || !ub || nx < 0 || ny < 0 || nz < 0)
        return set_err(MHD_ERR_ARG);
    const size_t cells = (size_t)nx * ny * nz;
    MHD_TRY(set_err(op_copy(c, u, uu, cells * 5 * c->elem)));
    return set_err(op_copy(c, b, ub, cells * 3 * c->elem));
}

static int read_clock(mhd_ctx* c, const void* clock, double out[4])
{
    if (c->elem == 4) {
        float h[4];
        CUDA_TRY(cudaMemcpyAsync(h, clock, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(cudaStreamSynchronize(c->stream));
        for (int s = 0; s < 4; s++)
            out[s] = h[s];
    } else {
        CUDA_TRY(cudaMemcpyAsync(out, clock, 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(cudaStreamSynchronize(c->stream));
    }
    return MHD_OK;
}

static int calcfl_sync(mhd_ctx* c, const void* u, const void* b, int nx, int ny, int nz, double* inv)
{
    const size_t cells = (size_t)nx * ny * nz;
    if (cells == 0) {  // the reference returns 1/0 with c = 0
        *inv = INFINITY;
        return MHD_OK;
    }
    int np = 0;
    MHD_TRY(c->opclock.ensure(4 * sizeof(double)));
    MHD_TRY(op_calcfl_partials(c, c->opart, u, b, cells, &np));
    MHD_TRY(op_finalize(c, c->opart.p, c->opclock.p, np, u, b, nx, ny, nz, 0.0, 0));
    double clk[4];
    MHD_TRY(read_clock(c, c->opclock.p, clk));
    *inv = clk[3];
    int herr = 0;
    CUDA_TRY(cudaMemcpy(&herr, c->err_dev, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr & DEVERR_NONFINITE) {
        CUDA_TRY(cudaMemsetAsync(c->err_dev, 0, sizeof(int), c->stream));
        CUDA_TRY(cudaStreamSynchronize(c->stream));
        return MHD_ERR_NONFINITE;
    }
    return MHD_OK;
}

extern "C" MHD_API int mhd_op_calcfl(mhd_ctx* c, const void* u, const void* b, int nx, int ny, int nz,
                                     double* inv_cmax)
{
    if (!c || !u || !b || !inv_cmax || nx < 0 || ny < 0 || nz < 0)
        return set_err(MHD_ERR_ARG);
    return set_err(calcfl_sync(c, u, b, nx, ny, nz, inv_cmax));
}

// ----------------------------------------------------------------- state

// The state's device buffers, allocated once: the ping-pong state, the CFL
// partials of both producers (the first CFL pass and the fluidx epilogue)
// and the side array, so that a captured step never allocates.
static int ensure_state(mhd_ctx* c)
{
    const size_t bu = ncell(c) * 5 * c->elem, bb = ncell(c) * 3 * c->elem;
    for (int v = 0; v < 2; v++) {
        MHD_TRY(c->U[v].ensure(bu));
        MHD_TRY(c->B[v].ensure(bb));
    }
    MHD_TRY(c->cflred.ensure((size_t)kCflReduceCtas * c->ks->part_bytes));
    if (c->elem == 4)  // the side array of the plain and fused steps
        MHD_TRY(c->W.ensure(ncell(c) * 2 * sizeof(float)));
    const size_t a = (ncell(c) + 255) / 256;
    const size_t f = fluidx_parts(c);
    MHD_TRY(c->part.ensure(((a > f ? a : f) + 1) * c->ks->part_bytes));
    return MHD_OK;
}

extern "C" MHD_API int mhd_set_state(mhd_ctx* c, const void* u, const void* b, int where)
{
    if (!c || !u || !b)
        return set_err(MHD_ERR_ARG);
    const size_t bu = ncell(c) * 5 * c->elem, bb = ncell(c) * 3 * c->elem;
    MHD_TRY(set_err(ensure_state(c)));
    (void)where;  // direction inferred from the pointers (unified addressing)
    const cudaMemcpyKind kind = cudaMemcpyDefault;
    if (cudaMemcpyAsync(c->U[0].p, u, bu, kind, c->stream) != cudaSuccess ||
        cudaMemcpyAsync(c->B[0].p, b, bb, kind, c->stream) != cudaSuccess)
        return set_err(MHD_ERR_CUDA);
    c->have_state = true;
    c->cfl_valid = false;
    return set_err(mhd_set_time(c, 0.0, INFINITY));
}

extern "C" MHD_API int mhd_get_state(mhd_ctx* c, void* u, void* b, int where)
{
    if (!c || !u || !b || !c->have_state)
        return set_err(MHD_ERR_ARG);
    const size_t bu = ncell(c) * 5 * c->elem, bb = ncell(c) * 3 * c->elem;
    (void)where;  // direction inferred from the pointers (unified addressing)
    const cudaMemcpyKind kind = cudaMemcpyDefault;
    if (cudaMemcpyAsync(u, c->U[0].p, bu, kind, c->stream) != cudaSuccess ||
        cudaMemcpyAsync(b, c->B[0].p, bb, kind, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
        return set_err(MHD_ERR_CUDA);
    return set_err(MHD_OK);
}

extern "C" MHD_API int mhd_state_ptrs(mhd_ctx* c, void** u, void** b)
{
    if (!c || !c->have_state)
        return set_err(MHD_ERR_ARG);
    if (u)
        *u = c->U[0].p;
    if (b)
        *b = c->B[0].p;
    return set_err(MHD_OK);
}

extern "C" MHD_API int mhd_clock_ptr(mhd_ctx* c, void** clock)
{
    if (!c || !clock || !c->clock.p)
        return set_err(MHD_ERR_ARG);
    *clock = c->clock.p;
    return set_err(MHD_OK);
}

extern "C" MHD_API int mhd_set_time(mhd_ctx* c, double t, double tf)
{
    if (!c)
        return set_err(MHD_ERR_ARG);
    if (c->elem == 4) {
        float h[2] = {(float)t, (float)tf};
        if (cudaMemcpyAsync(c->clock.p, h, sizeof(h), cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
            return set_err(MHD_ERR_CUDA);
    } else {
        double h[2] = {t, tf};
        if (cudaMemcpyAsync(c->clock.p, h, sizeof(h), cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
            return set_err(MHD_ERR_CUDA);
    }
    if (cudaMemsetAsync(c->nsteps_dev, 0, sizeof(long long), c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
        return set_err(MHD_ERR_CUDA);
    return set_err(MHD_OK);
}

extern "C" MHD_API int mhd_get_time(mhd_ctx* c, double* t, double* dt, long long* steps)
{
    if (!c)
        return set_err(MHD_ERR_ARG);
    double clk[4];
    MHD_TRY(set_err(read_clock(c, c->clock.p, clk)));
    if (t)
        *t = clk[0];
    if (dt)
        *dt = clk[2];
    if (steps) {
        if (cudaMemcpy(steps, c->nsteps_dev, sizeof(long long), cudaMemcpyDeviceToHost) != cudaSuccess)
            return set_err(MHD_ERR_CUDA);
    }
    return set_err(MHD_OK);
}

// ------------------------------------------------------------- the step

// Events of the copy stream: entry (the compute stream's queued work), b out,
// u out, done, then one per copy-in chunk.
enum { kCevEntry = 0, kCevOutB, kCevOutU, kCevDone, kCevChunk0 };
constexpr int kHostChunks = 8;  // copy-in chunks of a host-buffer step

// The last step of a host-buffer step copies the final b out as soon as the
// last advectbyzx has written it (field 1) and u after the last fluidx
// (field 0), on the copy stream: the b copy overlaps the last fluidx, which
// reads b but does not write it.  Planes k0 .. k0+nk-1 along z (nk 0: all).
// Nothing happens for other steps.
static int copy_out(mhd_ctx* c, int field, int k0 = 0, int nk = 0)
{
    void* dst = field ? c->out_b : c->out_u;
    if (!dst || c->capturing)
        return MHD_OK;
    cudaEvent_t e = c->cev[field ? kCevOutB : kCevOutU];
    CUDA_TRY(cudaEventRecord(e, c->stream));
    CUDA_TRY(cudaStreamWaitEvent(c->cstream, e, 0));
    const size_t per_plane = (size_t)c->nx * c->ny * (field ? 3 : 5) * c->elem;
    const size_t off = (size_t)k0 * per_plane, bytes = (nk ? (size_t)nk : (size_t)c->nz) * per_plane;
    const char* src = static_cast<const char*>(field ? c->B[0].p : c->U[0].p) + off;
    CUDA_TRY(cudaMemcpyAsync(static_cast<char*>(dst) + off, src, bytes, cudaMemcpyDefault, c->cstream));
    return MHD_OK;
}

// Sets the plane range of the operators enqueued while it lives.
struct SlabRange {
    mhd_ctx* c;
    SlabRange(mhd_ctx* ctx, int k0, int nk) : c(ctx)
    {
        c->slab_beg = k0;
        c->slab_count = nk;
    }
    ~SlabRange() { c->slab_beg = c->slab_count = 0; }
};

// Slabs of the fused step's tail in a host-buffer step: 8 (or 4) ranges of
// planes along z when the tail's kernels take them, else 1 (no slabs).
static int host_tail_slabs(const mhd_ctx* c, const void* Wy)
{
    if (!c->out_u || c->capturing || !Wy || !c->ks->tail_slabs_ok)
        return 1;
    for (int s : {8, 4})
        if (c->nz % s == 0 && c->ks->tail_slabs_ok(c->nx, c->ny, c->nz, c->nz / s))
            return s;
    return 1;
}

// One plain Strang step on (U0,B0) -> (U0,B0), C/mhd.c:62-118 with the
// copy_matrix calls replaced by ping-pong buffers.  Requires cfl_valid (the
// partials of the current state in c->part): the last fluidx of the step
// writes the partials of the next state in its epilogue.
static int enqueue_plain_step(mhd_ctx* c, double cfl)
{
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    void *U0 = c->U[0].p, *U1 = c->U[1].p, *B0 = c->B[0].p, *B1 = c->B[1].p;
    const void* dt = static_cast<char*>(c->clock.p) + 2 * c->elem;
    // the (rho, m_x) side array of a forward sweep's fluidx, read by the
    // advectbyzx launches right after it (8 instead of 20 bytes per cell)
    auto side = [&](int ax, int ay, int az) -> void* {
        const bool al = ((size_t)ax * 5 * c->elem) % 16 == 0 && ((size_t)ax * 3 * c->elem) % 16 == 0;
        return (c->W.p && c->ks->fluidx_writes_w(ax, ay, az, al ? 1 : 0)) ? c->W.p : nullptr;
    };
    MHD_TRY(op_finalize(c, c->part.p, c->clock.p, c->cfl_nparts, U0, B0, nx, ny, nz, cfl, 1));
    // x sweep
    void* W = side(nx, ny, nz);
    MHD_TRY(op_fluidx(c, U1, U0, B0, nx, ny, nz, 0, dt, nullptr, 0, W));
    MHD_TRY(op_advect(c, B1, B0, U1, B0, nx, ny, nz, 0, dt, 0, W));
    // y sweep
    MHD_TRY(op_transpose(c, 1, U0, B0, U1, B1, nx, ny, nz));
    W = side(ny, nx, nz);
    MHD_TRY(op_fluidx(c, U1, U0, B0, ny, nx, nz, 0, dt, nullptr, 0, W));
    MHD_TRY(op_advect(c, B1, B0, U1, B0, ny, nx, nz, 0, dt, 0, W));
    // z sweep
    MHD_TRY(op_transpose(c, 2, U0, B0, U1, B1, ny, nx, nz));
    W = side(nz, nx, ny);
    MHD_TRY(op_fluidx(c, U1, U0, B0, nz, nx, ny, 0, dt, nullptr, 0, W));
    MHD_TRY(op_advect(c, B1, B0, U1, B0, nz, nx, ny, 0, dt, 0, W));
    MHD_TRY(op_advect(c, B0, B1, U1, B1, nz, nx, ny, 0, dt, 0, W));
    MHD_TRY(op_fluidx(c, U0, U1, B0, nz, nx, ny, 0, dt, nullptr));
    // back (the transposes write the side array of their output for the advectbyzx after them)
    auto tside = [&](int axis, int ax, int ay, int az) -> void* {
        return (c->W.p && c->ks->transpose_writes_w(axis, ax, ay, az)) ? c->W.p : nullptr;
    };
    W = tside(2, nz, nx, ny);
    MHD_TRY(op_transpose(c, 2, U1, B1, U0, B0, nz, nx, ny, W));
    MHD_TRY(op_advect(c, B0, B1, U1, B1, ny, nx, nz, 0, dt, 0, W));
    MHD_TRY(op_fluidx(c, U0, U1, B0, ny, nx, nz, 0, dt, nullptr));
    // x again
    W = tside(1, ny, nx, nz);
    MHD_TRY(op_transpose(c, 1, U1, B1, U0, B0, ny, nx, nz, W));
    MHD_TRY(op_advect(c, B0, B1, U1, B1, nx, ny, nz, 0, dt, 0, W));
    MHD_TRY(copy_out(c, 1));
    // last fluidx with the calcfl epilogue for the next step
    const size_t nparts = fluidx_parts(c);
    if (c->part.cap < nparts * c->ks->part_bytes)  // sized by mhd_set_state
        return MHD_ERR_ARG;
    MHD_TRY(op_fluidx(c, U0, U1, B0, nx, ny, nz, 0, dt, c->part.p));
    MHD_TRY(copy_out(c, 0));
    c->cfl_nparts = (int)nparts;
    return MHD_OK;
}

// One fused Strang step on (U0,B0) -> (U0,B0): the same operator sequence
// as the plain step with every transpose removed; the sweeps along y and z
// read the untransposed state and see it in the transposed component order,
// so each operator computes what the plain step's operator computes on the
// transposed arrays, and the results are identical.
static int enqueue_fused_step(mhd_ctx* c, double cfl)
{
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    void *U0 = c->U[0].p, *U1 = c->U[1].p, *B0 = c->B[0].p, *B1 = c->B[1].p;
    const void* dt = static_cast<char*>(c->clock.p) + 2 * c->elem;
    // Every fluidx but the last writes the side array the advectbyzx after it
    // reads: rho and the momentum along that advectbyzx's sweep (1 m_x, 2 m_y,
    // 3 m_z), 8 instead of 20 bytes per cell.
    const bool al = ((size_t)nx * 5 * c->elem) % 16 == 0 && ((size_t)nx * 3 * c->elem) % 16 == 0;
    void* Wx = (c->W.p && c->ks->fluidx_writes_w(nx, ny, nz, al ? 1 : 0)) ? c->W.p : nullptr;
    void* Wy = (c->W.p && c->ks->sweep_writes_w(1, nx, ny, nz)) ? c->W.p : nullptr;
    void* Wz = (c->W.p && c->ks->sweep_writes_w(2, nx, ny, nz)) ? c->W.p : nullptr;
    MHD_TRY(op_finalize(c, c->part.p, c->clock.p, c->cfl_nparts, U0, B0, nx, ny, nz, cfl, 1));
    // x
    MHD_TRY(op_fluidx(c, U1, U0, B0, nx, ny, nz, 0, dt, nullptr, 0, Wx));
    MHD_TRY(op_advect(c, B1, B0, U1, B0, nx, ny, nz, 0, dt, 0, Wx));
    // y
    MHD_TRY(op_fluidx(c, U0, U1, B1, nx, ny, nz, 0, dt, nullptr, 1, Wy, 2));
    MHD_TRY(op_advect(c, B0, B1, U0, B1, nx, ny, nz, 0, dt, 1, Wy));
    // z, z
    MHD_TRY(op_fluidx(c, U1, U0, B0, nx, ny, nz, 0, dt, nullptr, 2, Wz, 3));
    MHD_TRY(op_advect(c, B1, B0, U1, B0, nx, ny, nz, 0, dt, 2, Wz));
    MHD_TRY(op_advect(c, B0, B1, U1, B1, nx, ny, nz, 0, dt, 2, Wz));
    MHD_TRY(op_fluidx(c, U0, U1, B0, nx, ny, nz, 0, dt, nullptr, 2, Wz, 2));
    // y
    MHD_TRY(op_advect(c, B1, B0, U0, B0, nx, ny, nz, 0, dt, 1, Wz));
    const size_t nparts = fluidx_parts(c);
    if (c->part.cap < nparts * c->ks->part_bytes)
        return MHD_ERR_ARG;
    const int S = host_tail_slabs(c, Wy);
    if (S > 1) {
        // The last step of a host-buffer step: the y fluidx, the x advectbyzx
        // and the x fluidx run on S slabs of planes along z, and each slab's
        // b and u go out as soon as they are final.  The advectbyzx of planes
        // k0..k1-1 reads its inputs at k0-1 .. k1 (C/advectbyzxB1.c: u at k-1;
        // C/advectbyzxB2.c: b(1) at k takes the flux of plane k+1), and the
        // x fluidx reads b at k1: the y fluidx runs one slab ahead (its last
        // slab first, for the periodic neighbour of plane 0) and the x fluidx
        // one slab behind the advectbyzx.
        const int kc = nz / S;
        auto yfluidx = [&](int s) {
            SlabRange r(c, s * kc, kc);
            return op_fluidx(c, U1, U0, B1, nx, ny, nz, 0, dt, nullptr, 1, Wy, 1);
        };
        auto xfluidx = [&](int s) {
            {
                SlabRange r(c, s * kc, kc);
                MHD_TRY(op_fluidx(c, U0, U1, B0, nx, ny, nz, 0, dt, c->part.p, 0));
            }
            return copy_out(c, 0, s * kc, kc);
        };
        MHD_TRY(yfluidx(S - 1));
        MHD_TRY(yfluidx(0));
        for (int s = 0; s < S; s++) {
            if (s + 1 < S - 1)
                MHD_TRY(yfluidx(s + 1));
            {
                SlabRange r(c, s * kc, kc);
                MHD_TRY(op_advect(c, B0, B1, U1, B1, nx, ny, nz, 0, dt, 0, Wy));
            }
            MHD_TRY(copy_out(c, 1, s * kc, kc));
            if (s > 0)
                MHD_TRY(xfluidx(s - 1));
        }
        MHD_TRY(xfluidx(S - 1));
        c->cfl_nparts = (int)nparts;
        return MHD_OK;
    }
    MHD_TRY(op_fluidx(c, U1, U0, B1, nx, ny, nz, 0, dt, nullptr, 1, Wy, 1));
    // x, with the calcfl epilogue for the next step
    MHD_TRY(op_advect(c, B0, B1, U1, B1, nx, ny, nz, 0, dt, 0, Wy));
    MHD_TRY(copy_out(c, 1));
    MHD_TRY(op_fluidx(c, U0, U1, B0, nx, ny, nz, 0, dt, c->part.p, 0));
    MHD_TRY(copy_out(c, 0));
    c->cfl_nparts = (int)nparts;
    return MHD_OK;
}

static int enqueue_step(mhd_ctx* c, double cfl, int variant)
{
    return variant == MHD_FUSED ? enqueue_fused_step(c, cfl) : enqueue_plain_step(c, cfl);
}

static int ensure_cfl(mhd_ctx* c)
{
    if (c->cfl_valid)
        return MHD_OK;
    const size_t cells = ncell(c);
    int np = 0;
    MHD_TRY(op_calcfl_partials(c, c->part, c->U[0].p, c->B[0].p, cells, &np));
    c->cfl_nparts = np;
    c->cfl_valid = true;
    return MHD_OK;
}

static int step_once_direct(mhd_ctx* c, double cfl, int variant)
{
    MHD_TRY(ensure_cfl(c));
    MHD_TRY(enqueue_step(c, cfl, variant));
    return MHD_OK;
}

static int step_graph(mhd_ctx* c, double cfl, int variant)
{
    MHD_TRY(ensure_cfl(c));
    // The graph's first node (finalize) reads cfl_nparts partials; those are
    // written by the previous step's last fluidx, whose grid does not change.
    const int steady = (int)fluidx_parts(c);
    if (c->cfl_nparts != steady)  // first step after a standalone calcfl
        return step_once_direct(c, cfl, variant);
    if (!c->gexec[variant] || c->gcfl[variant] != cfl || c->gtune[variant] != tune_generation()) {
        if (c->gexec[variant]) {
            cudaGraphExecDestroy(c->gexec[variant]);
            c->gexec[variant] = nullptr;
        }
        cudaGraph_t g = nullptr;
        CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        c->capturing = true;
        const long long before = c->launch_count;
        int s = enqueue_step(c, cfl, variant);
        c->capturing = false;
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        c->launch_count = before;  // counted per replay below
        if (s != MHD_OK) {
            if (g)
                cudaGraphDestroy(g);
            return s;
        }
        CUDA_TRY(e);
        size_t nnodes = 0;
        cudaGraphGetNodes(g, nullptr, &nnodes);
        c->glaunches[variant] = (int)nnodes;
        e = cudaGraphInstantiate(&c->gexec[variant], g, 0);
        cudaGraphDestroy(g);
        CUDA_TRY(e);
        c->gcfl[variant] = cfl;
        c->gtune[variant] = tune_generation();
    }
    CUDA_TRY(cudaGraphLaunch(c->gexec[variant], c->stream));
    c->launch_count += c->glaunches[variant];
    return MHD_OK;
}

// The grid and variant checks of a step.
static int check_step(const mhd_ctx* c, int variant)
{
    if (variant == MHD_PLAIN && c->ny != c->nz)  // transpose13 is applied to (ny,nx,nz) and (nz,nx,ny)
        return MHD_ERR_UNSUPPORTED;
    if (variant == MHD_FUSED && !c->ks->fused_ok(c->nx, c->ny, c->nz))
        return MHD_ERR_UNSUPPORTED;
    MHD_TRY(check_dims(c->nx, c->ny, c->nz));
    MHD_TRY(check_dims(c->ny, c->nx, c->nz));
    MHD_TRY(check_dims(c->nz, c->nx, c->ny));
    return MHD_OK;
}

extern "C" MHD_API int mhd_step(mhd_ctx* c, int nsteps, double cfl, int variant)
{
    if (!c || !c->have_state || nsteps < 0 || !(cfl > 0) || (variant != MHD_PLAIN && variant != MHD_FUSED))
        return set_err(MHD_ERR_ARG);
    MHD_TRY(set_err(check_step(c, variant)));
    for (int s = 0; s < nsteps; s++) {
        int st = (c->use_graphs && !c->profile) ? step_graph(c, cfl, variant) : step_once_direct(c, cfl, variant);
        if (st != MHD_OK)
            return set_err(st);
    }
    return set_err(MHD_OK);
}

static int ensure_copy_stream(mhd_ctx* c)
{
    if (!c->cstream)
        CUDA_TRY(cudaStreamCreateWithFlags(&c->cstream, cudaStreamNonBlocking));
    while ((int)c->cev.size() < kCevChunk0 + kHostChunks) {
        cudaEvent_t e = nullptr;
        CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        c->cev.push_back(e);
    }
    return MHD_OK;
}

// Steps on a host-resident state (the reference's loop, C/mhd.c:59-124, with
// its arrays in host memory): u and b are copied in, stepped nsteps times and
// the result is copied back into them; the call returns when it is there.
// The copies overlap the step: the state comes in as kHostChunks chunks on a
// copy stream and the compute stream runs the first CFL pass of each chunk
// as it lands; the final b goes out while the last fluidx runs.  The
// context's clock is kept (the state is assumed to be at its time t).
extern "C" MHD_API int mhd_step_host(mhd_ctx* c, void* u, void* b, int nsteps, double cfl, int variant)
{
    if (!c || !u || !b || nsteps < 1 || !(cfl > 0) || (variant != MHD_PLAIN && variant != MHD_FUSED))
        return set_err(MHD_ERR_ARG);
    MHD_TRY(set_err(check_step(c, variant)));
    MHD_TRY(set_err(ensure_state(c)));
    MHD_TRY(set_err(ensure_copy_stream(c)));
    if (!c->have_state)
        MHD_TRY(mhd_set_time(c, 0.0, INFINITY));
    const size_t cells = ncell(c), eu = 5 * (size_t)c->elem, eb = 3 * (size_t)c->elem;
    char* U0 = static_cast<char*>(c->U[0].p);
    char* B0 = static_cast<char*>(c->B[0].p);
    const char* hu = static_cast<const char*>(u);
    const char* hb = static_cast<const char*>(b);
    // the copies start after the work already queued on the compute stream
    if (cudaEventRecord(c->cev[kCevEntry], c->stream) != cudaSuccess ||
        cudaStreamWaitEvent(c->cstream, c->cev[kCevEntry], 0) != cudaSuccess)
        return set_err(MHD_ERR_CUDA);
    // chunks of whole CFL partials (256 cells), so chunk k's partials follow chunk k-1's
    size_t chunk = (cells + kHostChunks - 1) / kHostChunks;
    chunk = (chunk + 255) / 256 * 256;
    for (int k = 0; k < kHostChunks; k++) {
        const size_t c0 = (size_t)k * chunk;
        if (c0 >= cells)
            break;
        const size_t n = (cells - c0 < chunk) ? cells - c0 : chunk;
        if (cudaMemcpyAsync(U0 + c0 * eu, hu + c0 * eu, n * eu, cudaMemcpyDefault, c->cstream) != cudaSuccess ||
            cudaMemcpyAsync(B0 + c0 * eb, hb + c0 * eb, n * eb, cudaMemcpyDefault, c->cstream) != cudaSuccess ||
            cudaEventRecord(c->cev[kCevChunk0 + k], c->cstream) != cudaSuccess ||
            cudaStreamWaitEvent(c->stream, c->cev[kCevChunk0 + k], 0) != cudaSuccess)
            return set_err(MHD_ERR_CUDA);
        int np = 0;
        KTimer kt(c, MHD_K_CALCFL);
        if (c->ks->calcfl(U0 + c0 * eu, B0 + c0 * eb, n, c0,
                          static_cast<char*>(c->part.p) + (c0 / 256) * c->ks->part_bytes, &np, BoxStrides{},
                          c->stream) != cudaSuccess)
            return set_err(MHD_ERR_CUDA);
    }
    c->cfl_nparts = (int)((cells + 255) / 256);
    c->cfl_valid = true;
    c->have_state = true;
    int st = MHD_OK;
    for (int s = 0; s < nsteps && st == MHD_OK; s++) {
        if (s + 1 == nsteps) {  // the last step copies its result out as it is produced
            c->out_u = u;
            c->out_b = b;
            st = step_once_direct(c, cfl, variant);
            c->out_u = c->out_b = nullptr;
        } else {
            st = (c->use_graphs && !c->profile) ? step_graph(c, cfl, variant) : step_once_direct(c, cfl, variant);
        }
    }
    // later work on the compute stream waits for the copies out
    const bool ok = cudaEventRecord(c->cev[kCevDone], c->cstream) == cudaSuccess &&
                    cudaStreamWaitEvent(c->stream, c->cev[kCevDone], 0) == cudaSuccess;
    const bool synced = cudaStreamSynchronize(c->cstream) == cudaSuccess;
    if (st != MHD_OK)
        return set_err(st);
    return set_err((ok && synced) ? MHD_OK : MHD_ERR_CUDA);
}

extern "C" MHD_API int mhd_use_graphs(mhd_ctx* c, int enable)
{
    if (!c)
        return set_err(MHD_ERR_ARG);
    c->use_graphs = enable ? 1 : 0;
    if (!enable)
        invalidate_graphs(c);
    return set_err(MHD_OK);
}

extern "C" MHD_API int mhd_check(mhd_ctx* c)
{
    if (!c)
        return set_err(MHD_ERR_ARG);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess)
        return set_err(MHD_ERR_CUDA);
    int herr = 0;
    if (cudaMemcpy(&herr, c->err_dev, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return set_err(MHD_ERR_CUDA);
    if (herr & DEVERR_TIMEOUT)
        return set_err(MHD_ERR_TIMEOUT);
    if (herr & DEVERR_NONFINITE)
        return set_err(MHD_ERR_NONFINITE);
    return set_err(MHD_OK);
}

extern "C" MHD_API int mhd_clear_errors(mhd_ctx* c)
{
    if (!c)
        return set_err(MHD_ERR_ARG);
    if (cudaMemsetAsync(c->err_dev, 0, sizeof(int), c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
        return set_err(MHD_ERR_CUDA);
    return set_err(MHD_OK);
}

// Self-test of the bounded waits: one warp waits on an mbarrier that expects
// one arrival which nothing makes.  After `limit` SM cycles the wait gives up,
// the kernel records DEVERR_TIMEOUT in the context's error word and returns.
__global__ void k_wait_selftest(int* err, long long limit)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0)
        mbar_init(&bar, 1);
    __syncwarp();
    mbar_wait_limit(&bar, 0, threadIdx.x == 0 ? err : nullptr, limit);
}

extern "C" MHD_API int mhd_selftest_wait(mhd_ctx* c, double seconds)
{
    if (!c || !(seconds > 0.0) || seconds > 2.0)
        return set_err(MHD_ERR_ARG);
    int dev = 0, khz = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev) != cudaSuccess)
        return set_err(MHD_ERR_CUDA);
    const long long limit = (long long)(seconds * 1e3 * (double)(khz > 0 ? khz : 2000000));
    k_wait_selftest<<<1, 32, 0, c->stream>>>(c->err_dev, limit);
    CUDA_TRY(cudaGetLastError());
    c->launch_count++;
    return set_err(MHD_OK);
}

// -------------------------------------------------------------- profiling

extern "C" MHD_API int mhd_profile(mhd_ctx* c, int enable)
{
    if (!c)
        return set_err(MHD_ERR_ARG);
    drain_profile(c);
    c->profile = enable ? 1 : 0;
    return set_err(MHD_OK);
}

extern "C" MHD_API int mhd_profile_read(mhd_ctx* c, int kernel, double* total_ms, long long* launches)
{
    if (!c || kernel < 0 || kernel >= MHD_K_COUNT)
        return set_err(MHD_ERR_ARG);
    drain_profile(c);
    if (total_ms)
        *total_ms = c->total_ms[kernel];
    if (launches)
        *launches = c->nlaunch[kernel];
    return set_err(MHD_OK);
}

extern "C" MHD_API int mhd_profile_reset(mhd_ctx* c)
{
    if (!c)
        return set_err(MHD_ERR_ARG);
    drain_profile(c);
    for (int k = 0; k < MHD_K_COUNT; k++) {
        c->total_ms[k] = 0;
        c->nlaunch[k] = 0;
    }
    return set_err(MHD_OK);
}

extern "C" MHD_API long long mhd_launch_count(mhd_ctx* c) { return c ? c->launch_count : -1; }

// ------------------------------------------------------------------ tuning

static std::atomic<int> g_tune[TUNE_COUNT];
static std::atomic<long long> g_tune_gen{0};

int mhd::tune_value(int key) { return (key >= 0 && key < TUNE_COUNT) ? g_tune[key].load() : 0; }
long long mhd::tune_generation() { return g_tune_gen.load(); }

static int tune_key(const char* key)
{
    static const char* names[TUNE_COUNT] = {"fluidx.threads", "advect.cells", "advect.slots", "advect.J", "advect.K",
                                            "fluidx.cells", "advect.kernel", "advect.xk", "sweep.kernel",
                                            "sweep.k", "sweep.slots"};
    if (!key)
        return -1;
    for (int k = 0; k < TUNE_COUNT; k++)
        if (strcmp(key, names[k]) == 0)
            return k;
    return -1;
}

int mhd::tune_index(const char* key) { return tune_key(key); }

int mhd::tune_swap(int key, int value)
{
    if (key < 0 || key >= TUNE_COUNT)
        return 0;
    return g_tune[key].exchange(value);
}

extern "C" MHD_API int mhd_tune_set(const char* key, int value)
{
    const int k = tune_key(key);
    if (k < 0 || value < 0)
        return set_err(MHD_ERR_ARG);
    g_tune[k].store(value);
    g_tune_gen.fetch_add(1);
    return set_err(MHD_OK);
}

extern "C" MHD_API int mhd_tune_get(const char* key)
{
    const int k = tune_key(key);
    return (k < 0) ? -1 : g_tune[k].load();
}

extern "C" MHD_API int mhd_divb_max(mhd_ctx* c, double* out)
{
    if (!c || !out || !c->have_state)
        return set_err(MHD_ERR_ARG);
    const size_t cells = ncell(c);
    const int nparts = (int)((cells + 255) / 256);
    MHD_TRY(set_err(c->divb.ensure(nparts * sizeof(double))));
    int np = 0;
    c->launch_count++;
    if (c->ks->divb(c->B[0].p, c->nx, c->ny, c->nz, static_cast<double*>(c->divb.p), &np, c->stream) != cudaSuccess)
        return set_err(MHD_ERR_CUDA);
    std::vector<double> h(np);
    if (cudaMemcpyAsync(h.data(), c->divb.p, np * sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
        return set_err(MHD_ERR_CUDA);
    double m = 0;
    for (double v : h)
        m = v > m ? v : m;
    *out = m;
    return set_err(MHD_OK);
}

// ----------------------------------------------------------- diagnostics

// Per-block partials of the run diagnostics (MHD_DIAG_* order): min rho,
// min p, max |div B|, sum rho, sum |m|^2/(2 rho), sum |B_c|^2/2, sum E,
// max |v|, with B_c the cell-centred field (the mean of the two faces,
// C/fluidx.c:71-81) and p = (gamma - 1)(E - |m|^2/(2 rho) - |B_c|^2/2).
// FP64 accumulation; a NaN in rho or p propagates into the minima.
template <typename R>
__global__ void __launch_bounds__(256) k_diag(const R* __restrict__ u, const R* __restrict__ b, int nx, int ny,
                                              int nz, double* part)
{
    constexpr int NQ = 8;
    const double inf = __longlong_as_double(0x7ff0000000000000LL);
    double acc[NQ] = {inf, inf, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const size_t ncell = (size_t)nx * ny * nz;
    for (size_t cell = (size_t)blockIdx.x * blockDim.x + threadIdx.x; cell < ncell;
         cell += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(cell % nx), j = (int)((cell / nx) % ny), k = (int)(cell / ((size_t)nx * ny));
        const size_t ci = ((size_t)k * ny + j) * nx + ((i + 1 == nx) ? 0 : i + 1);
        const size_t cj = ((size_t)k * ny + ((j + 1 == ny) ? 0 : j + 1)) * nx + i;
        const size_t ck = ((size_t)((k + 1 == nz) ? 0 : k + 1) * ny + j) * nx + i;
        const double rho = (double)u[cell * 5], mx = (double)u[cell * 5 + 1], my = (double)u[cell * 5 + 2];
        const double mz = (double)u[cell * 5 + 3], e = (double)u[cell * 5 + 4];
        const double b0 = (double)b[cell * 3], b1 = (double)b[cell * 3 + 1], b2 = (double)b[cell * 3 + 2];
        const double bx = 0.5 * (b0 + (double)b[ci * 3]), by = 0.5 * (b1 + (double)b[cj * 3 + 1]);
        const double bz = 0.5 * (b2 + (double)b[ck * 3 + 2]);
        const double m2 = mx * mx + my * my + mz * mz;
        const double ek = 0.5 * m2 / rho, em = 0.5 * (bx * bx + by * by + bz * bz);
        const double p = (5.0 / 3.0 - 1.0) * (e - ek - em);
        const double div = fabs(((double)b[ci * 3] - b0) + ((double)b[cj * 3 + 1] - b1) + ((double)b[ck * 3 + 2] - b2));
        acc[0] = (rho < acc[0] || rho != rho) ? rho : acc[0];
        acc[1] = (p < acc[1] || p != p) ? p : acc[1];
        acc[2] = fmax(acc[2], div);
        acc[3] += rho;
        acc[4] += ek;
        acc[5] += em;
        acc[6] += e;
        acc[7] = fmax(acc[7], sqrt(m2) / rho);
    }
    __shared__ double red[NQ][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        double x = acc[q];
        for (int o = 16; o > 0; o >>= 1) {
            const double y = __shfl_xor_sync(0xffffffffu, x, o);
            if (q < 2)
                x = (y < x || y != y) ? y : x;
            else if (q == 2 || q == 7)
                x = fmax(x, y);
            else
                x += y;
        }
        if (lane == 0)
            red[q][warp] = x;
    }
    __syncthreads();
    if (threadIdx.x < NQ) {
        const int q = threadIdx.x;
        double x = red[q][0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
            const double y = red[q][w];
            if (q < 2)
                x = (y < x || y != y) ? y : x;
            else if (q == 2 || q == 7)
                x = fmax(x, y);
            else
                x += y;
        }
        part[(size_t)blockIdx.x * NQ + q] = x;
    }
}

extern "C" MHD_API int mhd_diagnostics(mhd_ctx* c, double* out)
{
    if (!c || !out || !c->have_state)
        return set_err(MHD_ERR_ARG);
    constexpr int NQ = MHD_DIAG_COUNT;
    const size_t cells = ncell(c);
    int blocks = (int)((cells + 255) / 256);
    if (blocks > 1024)
        blocks = 1024;
    MHD_TRY(set_err(c->divb.ensure((size_t)blocks * NQ * sizeof(double))));
    double* part = static_cast<double*>(c->divb.p);
    if (c->elem == 4)
        k_diag<float><<<blocks, 256, 0, c->stream>>>(static_cast<const float*>(c->U[0].p),
                                                     static_cast<const float*>(c->B[0].p), c->nx, c->ny, c->nz, part);
    else
        k_diag<double><<<blocks, 256, 0, c->stream>>>(static_cast<const double*>(c->U[0].p),
                                                      static_cast<const double*>(c->B[0].p), c->nx, c->ny, c->nz, part);
    CUDA_TRY(cudaGetLastError());
    c->launch_count++;
    std::vector<double> h((size_t)blocks * NQ);
    if (cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
        return set_err(MHD_ERR_CUDA);
    for (int q = 0; q < NQ; q++) {
        double x = h[q];
        for (int blk = 1; blk < blocks; blk++) {
            const double y = h[(size_t)blk * NQ + q];
            if (q < 2)
                x = (y < x || y != y) ? y : x;
            else if (q == MHD_DIAG_MAX_DIVB || q == MHD_DIAG_MAX_SPEED)
                x = y > x ? y : x;
            else
                x += y;
        }
        out[q] = x;
    }
    return set_err(MHD_OK);
}

// ----------------------------------------------------------- drop-in layer

static std::mutex g_dropin_mu;
static mhd_ctx* g_dropin = nullptr;
static int g_dropin_mode = -1;

static int dropin_ctx(mhd_ctx** out)
{
    if (g_dropin_mode < 0) {
        const char* m = getenv("MHD_GB300_MODE");
        g_dropin_mode = (m && (strcmp(m, "exact") == 0 || strcmp(m, "EXACT") == 0)) ? MHD_MODE_EXACT : MHD_MODE_FAST;
    }
    if (!g_dropin) {
        int s = mhd_create(&g_dropin, 1, 1, 1, MHD_F32 | g_dropin_mode);
        if (s != MHD_OK)
            return s;
    }
    *out = g_dropin;
    return MHD_OK;
}

extern "C" MHD_API int mhd_set_dropin_mode(int mode)
{
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    if (mode != MHD_MODE_FAST && mode != MHD_MODE_EXACT)
        return set_err(MHD_ERR_ARG);
    g_dropin_mode = mode;
    if (g_dropin) {
        g_dropin->flags = MHD_F32 | mode;
        g_dropin->ks = pick_set(g_dropin->flags);
    }
    return set_err(MHD_OK);
}

// A drop-in argument: device-accessible pointers are used in place; host
// memory is staged through a cached device mirror (copied in if read, copied
// back if written).
struct Arg {
    void* user;
    size_t bytes;
    bool in, out;
    void* dev = nullptr;
    bool staged = false;
};

static bool device_accessible(const void* p)
{
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

static int stage_in(mhd_ctx* c, Arg* args, int na)
{
    int slot = 0;
    for (int s = 0; s < na; s++) {
        Arg& a = args[s];
        // the same user pointer twice shares one mirror
        for (int t = 0; t < s; t++)
            if (args[t].user == a.user && args[t].bytes == a.bytes) {
                a.dev = args[t].dev;
                a.staged = args[t].staged;
                break;
            }
        if (a.dev)
            continue;
        if (device_accessible(a.user)) {
            a.dev = a.user;
            continue;
        }
        MHD_TRY(c->stage[slot].ensure(a.bytes));
        a.dev = c->stage[slot].p;
        a.staged = true;
        slot++;
        if (a.in)
            CUDA_TRY(cudaMemcpyAsync(a.dev, a.user, a.bytes, cudaMemcpyHostToDevice, c->stream));
    }
    return MHD_OK;
}

static int stage_out(mhd_ctx* c, Arg* args, int na)
{
    for (int s = 0; s < na; s++) {
        Arg& a = args[s];
        bool first = true;
        for (int t = 0; t < s; t++)
            if (args[t].user == a.user && args[t].out)
                first = false;
        if (a.staged && a.out && first)
            CUDA_TRY(cudaMemcpyAsync(a.user, a.dev, a.bytes, cudaMemcpyDeviceToHost, c->stream));
    }
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return MHD_OK;
}

static bool dims_ok(const int* nx, const int* ny, const int* nz)
{
    return nx && ny && nz && *nx >= 0 && *ny >= 0 && *nz >= 0;
}

static size_t cells_of(const int* nx, const int* ny, const int* nz) { return (size_t)(*nx) * (*ny) * (*nz); }

extern "C" MHD_API void fluidx(float* u, float* b, int* nx, int* ny, int* nz, float* dt, float* update_u,
                               float* update_b, int iter)
{
    (void)b;
    (void)iter;
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    if (!u || !update_u || !update_b || !dt || !dims_ok(nx, ny, nz)) {
        set_err(MHD_ERR_ARG);
        return;
    }
    const size_t cells = cells_of(nx, ny, nz);
    if (cells == 0) {
        set_err(MHD_OK);
        return;
    }
    mhd_ctx* c;
    if (set_err(dropin_ctx(&c)) != MHD_OK)
        return;
    Arg args[3] = {{update_u, cells * 20, true, false}, {update_b, cells * 12, true, false}, {u, cells * 20, false, true}};
    if (set_err(stage_in(c, args, 3)) != MHD_OK)
        return;
    if (set_err(op_fluidx(c, args[2].dev, args[0].dev, args[1].dev, *nx, *ny, *nz, (double)*dt, nullptr, nullptr)) !=
        MHD_OK)
        return;
    set_err(stage_out(c, args, 3));
}

extern "C" MHD_API void advectbyzx(float* u, float* b, int* nx, int* ny, int* nz, float* dt, float* update_u,
                                   float* update_b)
{
    (void)u;
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    if (!b || !update_u || !update_b || !dt || !dims_ok(nx, ny, nz)) {
        set_err(MHD_ERR_ARG);
        return;
    }
    const size_t cells = cells_of(nx, ny, nz);
    if (cells == 0) {
        set_err(MHD_OK);
        return;
    }
    mhd_ctx* c;
    if (set_err(dropin_ctx(&c)) != MHD_OK)
        return;
    Arg args[3] = {{update_u, cells * 20, true, false}, {update_b, cells * 12, true, false}, {b, cells * 12, true, true}};
    if (set_err(stage_in(c, args, 3)) != MHD_OK)
        return;
    const void* ub = args[1].dev;
    if (args[2].dev == ub) {  // b and update_b alias: keep a private copy of the input
        if (set_err(c->alias[1].ensure(cells * 12)) != MHD_OK || set_err(op_copy(c, ub, c->alias[1].p, cells * 12)) != MHD_OK)
            return;
        ub = c->alias[1].p;
    }
    if (set_err(op_advect(c, args[2].dev, args[2].dev, args[0].dev, ub, *nx, *ny, *nz, (double)*dt, nullptr)) !=
        MHD_OK)
        return;
    set_err(stage_out(c, args, 3));
}

static void dropin_transpose(int axis, float* u, float* b, float* update_u, float* update_b, int* nx, int* ny, int* nz)
{
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    if (!u || !b || !update_u || !update_b || !dims_ok(nx, ny, nz)) {
        set_err(MHD_ERR_ARG);
        return;
    }
    if (axis == 2 && *nx != *nz) {  // C/transpose13.c:50-61 leaves the outputs untouched
        set_err(MHD_ERR_ARG);
        return;
    }
    const size_t cells = cells_of(nx, ny, nz);
    if (cells == 0) {
        set_err(MHD_OK);
        return;
    }
    mhd_ctx* c;
    if (set_err(dropin_ctx(&c)) != MHD_OK)
        return;
    Arg args[4] = {{update_u, cells * 20, true, false},
                   {update_b, cells * 12, true, false},
                   {u, cells * 20, false, true},
                   {b, cells * 12, false, true}};
    if (set_err(stage_in(c, args, 4)) != MHD_OK)
        return;
    if (set_err(transpose_entry(c, axis, args[2].dev, args[3].dev, args[0].dev, args[1].dev, *nx, *ny, *nz)) != MHD_OK)
        return;
    set_err(stage_out(c, args, 4));
}

extern "C" MHD_API void transpose12(float* u, float* b, float* update_u, float* update_b, int* nx, int* ny, int* nz,
                                    int iter)
{
    (void)iter;
    dropin_transpose(1, u, b, update_u, update_b, nx, ny, nz);
}

extern "C" MHD_API void transpose13(float* u, float* b, float* update_u, float* update_b, int* nx, int* ny, int* nz)
{
    dropin_transpose(2, u, b, update_u, update_b, nx, ny, nz);
}

extern "C" MHD_API void copy_matrix(float* u, float* b, int* nx, int* ny, int* nz, float* update_u, float* update_b)
{
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    if (!u || !b || !update_u || !update_b || !dims_ok(nx, ny, nz)) {
        set_err(MHD_ERR_ARG);
        return;
    }
    const size_t cells = cells_of(nx, ny, nz);
    if (cells == 0) {
        set_err(MHD_OK);
        return;
    }
    mhd_ctx* c;
    if (set_err(dropin_ctx(&c)) != MHD_OK)
        return;
    Arg args[4] = {{u, cells * 20, true, false},
                   {b, cells * 12, true, false},
                   {update_u, cells * 20, false, true},
                   {update_b, cells * 12, false, true}};
    if (set_err(stage_in(c, args, 4)) != MHD_OK)
        return;
    if (set_err(op_copy(c, args[0].dev, args[2].dev, cells * 20)) != MHD_OK ||
        set_err(op_copy(c, args[1].dev, args[3].dev, cells * 12)) != MHD_OK)
        return;
    set_err(stage_out(c, args, 4));
}

extern "C" MHD_API float calcfl(float* u, float* b, int* nx, int* ny, int* nz)
{
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    if (!u || !b || !dims_ok(nx, ny, nz)) {
        set_err(MHD_ERR_ARG);
        return NAN;
    }
    const size_t cells = cells_of(nx, ny, nz);
    if (cells == 0) {
        set_err(MHD_OK);
        return INFINITY;
    }
    mhd_ctx* c;
    if (set_err(dropin_ctx(&c)) != MHD_OK)
        return NAN;
    Arg args[2] = {{u, cells * 20, true, false}, {b, cells * 12, true, false}};
    if (set_err(stage_in(c, args, 2)) != MHD_OK)
        return NAN;
    double inv = NAN;
    int s = calcfl_sync(c, args[0].dev, args[1].dev, *nx, *ny, *nz, &inv);
    set_err(s);
    return (float)inv;
}

// ------------------------------------------------- CUDA-side compatibility names
//
// The reference's CUDA host code (Cuda/cuda_subroutine.h:4-12) calls these
// five names with device arrays, device copies of the dimensions (ignored
// here) and host copies (used).  They run this library's kernels with the
// C path's arithmetic (Cuda/ itself diverges from C/), on the drop-in
// context, and return after the work is done like the reference's
// cudaThreadSynchronize.

static bool host_dims_ok(const int* nx, const int* ny, const int* nz)
{
    return nx && ny && nz && *nx > 0 && *ny > 0 && *nz > 0;
}

// dt <- 1/max speed (Cuda/cuda_cfl.cu:14-45): *h_dt on the host and a copy in dt (device)
extern "C" MHD_API void cuda_cfl(float* u, float* b, int* nx, int* ny, int* nz, float* dt, float* c_scratch,
                                 int* h_nx, int* h_ny, int* h_nz, float* h_dt)
{
    (void)nx, (void)ny, (void)nz, (void)c_scratch;
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    if (!u || !b || !dt || !h_dt || !host_dims_ok(h_nx, h_ny, h_nz)) {
        set_err(MHD_ERR_ARG);
        return;
    }
    mhd_ctx* c;
    if (set_err(dropin_ctx(&c)) != MHD_OK)
        return;
    double inv = NAN;
    if (set_err(calcfl_sync(c, u, b, *h_nx, *h_ny, *h_nz, &inv)) != MHD_OK)
        return;
    *h_dt = (float)inv;
    set_err(cudaMemcpy(dt, h_dt, sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess ? MHD_OK : MHD_ERR_CUDA);
}

// u <- fluidx(u, b) in place, dt read on the device (Cuda/cuda_fluidx.cu:12-23)
extern "C" MHD_API void cuda_fluidx(float* u, float* b, int* nx, int* ny, int* nz, float* dt, int* h_nx, int* h_ny,
                                    int* h_nz)
{
    (void)nx, (void)ny, (void)nz;
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    if (!u || !b || !dt || !host_dims_ok(h_nx, h_ny, h_nz)) {
        set_err(MHD_ERR_ARG);
        return;
    }
    mhd_ctx* c;
    if (set_err(dropin_ctx(&c)) != MHD_OK)
        return;
    // in place is safe: a CTA reads only its own u pencils (and b)
    if (set_err(op_fluidx(c, u, u, b, *h_nx, *h_ny, *h_nz, 0.0, dt, nullptr)) != MHD_OK)
        return;
    set_err(cudaStreamSynchronize(c->stream) == cudaSuccess ? MHD_OK : MHD_ERR_CUDA);
}

// b <- advectbyzx(u, b) in place (Cuda/cuda_advectbyzx.cu); `temp` (the reference's EMF
// scratch) is not needed
extern "C" MHD_API void cuda_advectbyzx(float* u, float* b, int* nx, int* ny, int* nz, float* dt, float* temp,
                                        int* h_nx, int* h_ny, int* h_nz)
{
    (void)nx, (void)ny, (void)nz, (void)temp;
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    if (!u || !b || !dt || !host_dims_ok(h_nx, h_ny, h_nz)) {
        set_err(MHD_ERR_ARG);
        return;
    }
    mhd_ctx* c;
    if (set_err(dropin_ctx(&c)) != MHD_OK)
        return;
    const size_t bytes = (size_t)(*h_nx) * (*h_ny) * (*h_nz) * 12;
    // neighbouring rows of b are read while b is written: advect from a private copy
    if (set_err(c->alias[1].ensure(bytes)) != MHD_OK || set_err(op_copy(c, b, c->alias[1].p, bytes)) != MHD_OK)
        return;
    if (set_err(op_advect(c, b, c->alias[1].p, u, c->alias[1].p, *h_nx, *h_ny, *h_nz, 0.0, dt)) != MHD_OK)
        return;
    set_err(cudaStreamSynchronize(c->stream) == cudaSuccess ? MHD_OK : MHD_ERR_CUDA);
}

static void cuda_transpose(int axis, float* ut, float* bt, float* u, float* b, const int* h_nx, const int* h_ny,
                           const int* h_nz)
{
    std::lock_guard<std::mutex> lk(g_dropin_mu);
    if (!ut || !bt || !u || !b || !host_dims_ok(h_nx, h_ny, h_nz) || ut == u || bt == b) {
        set_err(MHD_ERR_ARG);
        return;
    }
    mhd_ctx* c;
    if (set_err(dropin_ctx(&c)) != MHD_OK)
        return;
    if (set_err(op_transpose(c, axis, ut, bt, u, b, *h_nx, *h_ny, *h_nz, nullptr, true)) != MHD_OK)
        return;
    // like the reference's wrappers (Cuda/cuda_transpose12.cu:30-34), the
    // transposed state is copied back, so u and b hold it on return as well
    const size_t cells = (size_t)(*h_nx) * (*h_ny) * (*h_nz);
    if (set_err(op_copy(c, ut, u, cells * 5 * sizeof(float))) != MHD_OK ||
        set_err(op_copy(c, bt, b, cells * 3 * sizeof(float))) != MHD_OK)
        return;
    set_err(cudaStreamSynchronize(c->stream) == cudaSuccess ? MHD_OK : MHD_ERR_CUDA);
}

// (ut, bt) <- transpose12(u, b), then (u, b) <- (ut, bt) (Cuda/cuda_transpose12.cu:12-38)
extern "C" MHD_API void cuda_transpose12(float* ut, float* bt, float* u, float* b, int* nx, int* ny, int* nz,
                                         int* h_nx, int* h_ny, int* h_nz)
{
    (void)nx, (void)ny, (void)nz;
    cuda_transpose(1, ut, bt, u, b, h_nx, h_ny, h_nz);
}

// (ut, bt) <- transpose13(u, b), then (u, b) <- (ut, bt); nx == nz, nz == 1 or nx == 1
// (Cuda/cuda_transpose13.cu:14-55)
extern "C" MHD_API void cuda_transpose13(float* ut, float* bt, float* u, float* b, int* nx, int* ny, int* nz,
                                         int* h_nx, int* h_ny, int* h_nz)
{
    (void)nx, (void)ny, (void)nz;
    cuda_transpose(2, ut, bt, u, b, h_nx, h_ny, h_nz);
}
