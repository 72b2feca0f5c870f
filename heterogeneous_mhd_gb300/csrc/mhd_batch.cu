// Batched boxes: many independent periodic cubes of uneven sizes advanced
// together, each with its own dt (the benchmarked workload: 256 boxes of
// edge 32..128).
//
// The boxes are grouped by edge length.  Each size class keeps its boxes'
// states contiguous (ping-pong pairs like the single-box context); each box
// has its own CFL partials, clock and dt.  The FP32 classes of edge 32, 48,
// 64, 96 and 128 (up to eight classes) step together by work-list launches:
// one launch per operator of the Strang step (C/mhd.c:62-118) walks the
// (class, box, tile) list of all of them (mhd_multi.cuh), 17 launches per
// step for the whole group.  Every other class, and every class given its own
// launch shapes (mhd_batch_tune_edge) or all classes when the work list is
// switched off (mhd_batch_set_worklist), takes one launch per operator with
// the box index in blockIdx.z (BoxStrides in mhd_kernels.cuh).  The whole
// step of every class is captured into one CUDA graph.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/mhd_gb300.h"
#include "mhd_launch.h"

using namespace mhd;

namespace {

struct SizeClass {
    int n = 0;
    std::vector<int> boxes;  // global box ids in class order
    void* U[2] = {nullptr, nullptr};
    void* B[2] = {nullptr, nullptr};
    void* clock = nullptr;  // per box R[4]: t, tf, dt, 1/c
    void* part = nullptr;   // per box CFL partials
    size_t part_per_box = 0;
    int cfl_nparts = 0;     // partials per box currently held
    size_t ustride = 0;     // bytes between consecutive boxes' u (256-byte aligned)
    size_t bstride = 0;
    void* W = nullptr;      // (rho, m_x) side arrays of the boxes, one after the other (FP32; classes
                            // whose own x-sweep advectbyzx reads it, KernelSet::batch_side_ok, and
                            // classes that can step in the work list, whose advectbyzx always reads it)
    int knobs[TUNE_COUNT];  // launch-shape knobs of this class's launches (-1: the global setting)
    bool multi = false;     // steps in the work-list launches (assign_worklist)
    bool side = false;      // its own launches use W (KernelSet::batch_side_ok)
    SizeClass() { std::fill(knobs, knobs + TUNE_COUNT, -1); }
    bool own_shapes() const
    {
        for (int k = 0; k < TUNE_COUNT; k++)
            if (knobs[k] >= 0)
                return true;
        return false;
    }
    size_t cells() const { return (size_t)n * n * n; }
};

// Applies a class's own launch-shape knobs for the duration of its enqueue
// and puts the global values back afterwards.
struct ClassKnobs {
    int saved[TUNE_COUNT];
    const SizeClass& c;
    explicit ClassKnobs(const SizeClass& cls) : c(cls)
    {
        for (int k = 0; k < TUNE_COUNT; k++)
            saved[k] = (c.knobs[k] >= 0) ? tune_swap(k, c.knobs[k]) : -1;
    }
    ~ClassKnobs()
    {
        for (int k = 0; k < TUNE_COUNT; k++)
            if (c.knobs[k] >= 0)
                tune_swap(k, saved[k]);
    }
};

static size_t round256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

struct mhd_batch {
    int flags = 0;
    const KernelSet* ks = nullptr;
    int elem = 4;
    cudaStream_t stream = nullptr;
    std::vector<SizeClass> cls;
    std::vector<std::pair<int, int>> where;  // box -> (class, index in class)
    std::vector<char> loaded;                // box state set by mhd_batch_set_box
    int* err_dev = nullptr;
    long long* nsteps_dev = nullptr;
    bool cfl_valid = false;
    cudaGraphExec_t graph = nullptr;
    double gcfl = 0;
    long long gtune = -1;
    int glaunches = 0;
    long long launches = 0;
    bool worklist = true;  // eligible classes step in work-list launches
};

static int cu(cudaError_t e) { return e == cudaSuccess ? MHD_OK : (e == cudaErrorMemoryAllocation ? MHD_ERR_NOMEM : MHD_ERR_CUDA); }

#define BTRY(x)                \
    do {                       \
        int s_ = (x);          \
        if (s_ != MHD_OK)      \
            return s_;         \
    } while (0)

static bool tma_ok(const mhd_batch* b, int n) { return ((size_t)n * 5 * b->elem) % 16 == 0 && ((size_t)n * 3 * b->elem) % 16 == 0; }

// a class that can step in the work-list launches (its launch shapes are then
// those of mhd_multi.cuh, so a class given its own shapes keeps its own launches)
static bool worklist_ok(const mhd_batch* b, const SizeClass& c)
{
    return b->worklist && b->elem == 4 && b->ks->multi_ok(c.n) && tma_ok(b, c.n) && c.W && !c.own_shapes();
}

// Marks the classes of the work-list group: the eligible ones, at most
// kMaxSegs of them (the largest by cells when there are more).
static void assign_worklist(mhd_batch* b)
{
    std::vector<int> ok;
    for (int i = 0; i < (int)b->cls.size(); i++) {
        b->cls[i].multi = false;
        if (worklist_ok(b, b->cls[i]))
            ok.push_back(i);
    }
    std::stable_sort(ok.begin(), ok.end(), [&](int x, int y) {
        return b->cls[x].cells() * b->cls[x].boxes.size() > b->cls[y].cells() * b->cls[y].boxes.size();
    });
    for (int k = 0; k < (int)ok.size() && k < kMaxSegs; k++)
        b->cls[ok[k]].multi = true;
}

// CFL partials per box that the step's last fluidx writes for a class
static int fluidx_parts_of(const mhd_batch* b, const SizeClass& c)
{
    return c.multi ? b->ks->multi_fluidx_parts(c.n) : b->ks->fluidx_parts(c.n, c.n, c.n, tma_ok(b, c.n));
}

static BoxStrides strides(const mhd_batch* b, const SizeClass& c)
{
    BoxStrides s;
    s.u = c.ustride;
    s.b = c.bstride;
    s.dt = 4 * (size_t)b->elem;
    s.w = c.W ? c.cells() * 8 : 0;
    s.count = (int)c.boxes.size();
    return s;
}

extern "C" MHD_API int mhd_batch_destroy(mhd_batch* b)
{
    if (!b)
        return MHD_ERR_ARG;
    cudaStreamSynchronize(b->stream);
    if (b->graph)
        cudaGraphExecDestroy(b->graph);
    for (auto& c : b->cls) {
        for (int v = 0; v < 2; v++) {
            cudaFree(c.U[v]);
            cudaFree(c.B[v]);
        }
        cudaFree(c.clock);
        cudaFree(c.part);
        cudaFree(c.W);
    }
    cudaFree(b->err_dev);
    if (b->stream)
        cudaStreamDestroy(b->stream);
    delete b;
    return MHD_OK;
}

extern "C" MHD_API int mhd_batch_create(mhd_batch** out, int nboxes, const int* sizes, int flags)
{
    if (!out || nboxes <= 0 || !sizes)
        return MHD_ERR_ARG;
    *out = nullptr;
    for (int i = 0; i < nboxes; i++)
        if (sizes[i] <= 0 || sizes[i] > 512)
            return MHD_ERR_ARG;
    mhd_batch* b = new mhd_batch();
    b->flags = flags;
    b->ks = (flags & MHD_F64) ? kernels_f64_exact() : ((flags & MHD_MODE_EXACT) ? kernels_f32_exact() : kernels_f32_fast());
    b->elem = b->ks->elem;
    // group by edge; a class holds at most 65535/n boxes (grid z of the transposes)
    std::map<int, std::vector<int>> by_edge;
    for (int i = 0; i < nboxes; i++)
        by_edge[sizes[i]].push_back(i);
    b->where.resize(nboxes);
    b->loaded.assign(nboxes, 0);
    for (auto& kv : by_edge) {
        const size_t cap = (size_t)(65535 / kv.first);
        for (size_t k = 0; k < kv.second.size(); k++) {
            if (k % cap == 0) {
                b->cls.emplace_back();
                b->cls.back().n = kv.first;
            }
            SizeClass& c = b->cls.back();
            b->where[kv.second[k]] = {(int)b->cls.size() - 1, (int)c.boxes.size()};
            c.boxes.push_back(kv.second[k]);
        }
    }
    int st = cu(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    if (st == MHD_OK)
        st = cu(cudaMalloc(&b->err_dev, 64));
    if (st == MHD_OK)
        st = cu(cudaMemset(b->err_dev, 0, 64));
    b->nsteps_dev = reinterpret_cast<long long*>(reinterpret_cast<char*>(b->err_dev) + 8);
    for (auto& c : b->cls) {
        if (st != MHD_OK)
            break;
        const size_t m = c.boxes.size();
        c.ustride = round256(c.cells() * 5 * b->elem);
        c.bstride = round256(c.cells() * 3 * b->elem);
        for (int v = 0; v < 2 && st == MHD_OK; v++) {
            st = cu(cudaMalloc(&c.U[v], m * c.ustride));
            if (st == MHD_OK)
                st = cu(cudaMalloc(&c.B[v], m * c.bstride));
        }
        // the (rho, m_x) side array: classes whose x-sweep advectbyzx reads it, and every class
        // that can step in the work-list launches (whose advectbyzx always reads it)
        c.side = b->elem == 4 && b->ks->batch_side_ok(c.n, (int)m);
        if (st == MHD_OK && (c.side || (b->elem == 4 && b->ks->multi_ok(c.n) && tma_ok(b, c.n))))
            st = cu(cudaMalloc(&c.W, m * c.cells() * 8));
        const size_t pa = (c.cells() + 255) / 256 + 1, pf = (size_t)b->ks->fluidx_parts(c.n, c.n, c.n, tma_ok(b, c.n));
        c.part_per_box = std::max(pa, pf);
        if (b->ks->multi_ok(c.n))
            c.part_per_box = std::max(c.part_per_box, (size_t)b->ks->multi_fluidx_parts(c.n));
        if (st == MHD_OK)
            st = cu(cudaMalloc(&c.part, m * c.part_per_box * b->ks->part_bytes));
        if (st == MHD_OK)
            st = cu(cudaMalloc(&c.clock, m * 4 * (size_t)b->elem));
        if (st == MHD_OK) {  // t = 0, tf = +inf for every box
            std::vector<double> h(4 * m);
            for (size_t i = 0; i < m; i++) {
                h[4 * i] = 0;
                h[4 * i + 1] = INFINITY;
                h[4 * i + 2] = 0;
                h[4 * i + 3] = 0;
            }
            if (b->elem == 4) {
                std::vector<float> hf(h.begin(), h.end());
                st = cu(cudaMemcpy(c.clock, hf.data(), hf.size() * 4, cudaMemcpyHostToDevice));
            } else {
                st = cu(cudaMemcpy(c.clock, h.data(), h.size() * 8, cudaMemcpyHostToDevice));
            }
        }
    }
    if (st != MHD_OK) {
        mhd_batch_destroy(b);
        return st;
    }
    *out = b;
    return MHD_OK;
}

extern "C" MHD_API int mhd_batch_set_box(mhd_batch* b, int box, const void* u, const void* bf, int where)
{
    (void)where;  // direction inferred from the pointers (unified addressing)
    if (!b || box < 0 || box >= (int)b->where.size() || !u || !bf)
        return MHD_ERR_ARG;
    SizeClass& c = b->cls[b->where[box].first];
    const size_t k = b->where[box].second;
    const size_t bu = c.cells() * 5 * b->elem, bb = c.cells() * 3 * b->elem;
    BTRY(cu(cudaMemcpyAsync(static_cast<char*>(c.U[0]) + k * c.ustride, u, bu, cudaMemcpyDefault, b->stream)));
    BTRY(cu(cudaMemcpyAsync(static_cast<char*>(c.B[0]) + k * c.bstride, bf, bb, cudaMemcpyDefault, b->stream)));
    if (b->elem == 4) {
        const float h[4] = {0.f, INFINITY, 0.f, 0.f};
        BTRY(cu(cudaMemcpyAsync(static_cast<char*>(c.clock) + k * 16, h, 16, cudaMemcpyHostToDevice, b->stream)));
    } else {
        const double h[4] = {0.0, INFINITY, 0.0, 0.0};
        BTRY(cu(cudaMemcpyAsync(static_cast<char*>(c.clock) + k * 32, h, 32, cudaMemcpyHostToDevice, b->stream)));
    }
    BTRY(cu(cudaStreamSynchronize(b->stream)));
    b->loaded[box] = 1;
    b->cfl_valid = false;
    return MHD_OK;
}

extern "C" MHD_API int mhd_batch_get_box(mhd_batch* b, int box, void* u, void* bf, int where)
{
    (void)where;
    if (!b || box < 0 || box >= (int)b->where.size() || !u || !bf)
        return MHD_ERR_ARG;
    SizeClass& c = b->cls[b->where[box].first];
    const size_t k = b->where[box].second;
    const size_t bu = c.cells() * 5 * b->elem, bb = c.cells() * 3 * b->elem;
    BTRY(cu(cudaMemcpyAsync(u, static_cast<char*>(c.U[0]) + k * c.ustride, bu, cudaMemcpyDefault, b->stream)));
    BTRY(cu(cudaMemcpyAsync(bf, static_cast<char*>(c.B[0]) + k * c.bstride, bb, cudaMemcpyDefault, b->stream)));
    return cu(cudaStreamSynchronize(b->stream));
}

extern "C" MHD_API int mhd_batch_time(mhd_batch* b, int box, double* t, double* dt)
{
    if (!b || box < 0 || box >= (int)b->where.size())
        return MHD_ERR_ARG;
    SizeClass& c = b->cls[b->where[box].first];
    const size_t k = b->where[box].second;
    double h[4];
    if (b->elem == 4) {
        float f[4];
        BTRY(cu(cudaMemcpyAsync(f, static_cast<char*>(c.clock) + k * 16, 16, cudaMemcpyDeviceToHost, b->stream)));
        BTRY(cu(cudaStreamSynchronize(b->stream)));
        for (int i = 0; i < 4; i++)
            h[i] = f[i];
    } else {
        BTRY(cu(cudaMemcpyAsync(h, static_cast<char*>(c.clock) + k * 32, 32, cudaMemcpyDeviceToHost, b->stream)));
        BTRY(cu(cudaStreamSynchronize(b->stream)));
    }
    if (t)
        *t = h[0];
    if (dt)
        *dt = h[2];
    return MHD_OK;
}

// ---------------------------------------------------------------- the step

static int cfl_first_pass(mhd_batch* b)
{
    for (auto& c : b->cls) {
        int np = 0;
        BTRY(cu(b->ks->calcfl(c.U[0], c.B[0], c.cells(), 0, c.part, &np, strides(b, c), b->stream)));
        c.cfl_nparts = np;
        b->launches++;
    }
    b->cfl_valid = true;
    return MHD_OK;
}

// One Strang step of every class: the classes outside the work list first
// (the sequence of enqueue_plain_step for a single box, each launch covering
// all boxes of the class), then the work-list group (enqueue_multi).
static int enqueue_multi(mhd_batch* b, double cfl);

static int enqueue_step(mhd_batch* b, double cfl)
{
    assign_worklist(b);
    for (auto& c : b->cls) {
        if (c.multi)
            continue;
        const ClassKnobs knobs(c);
        const int n = c.n;
        const BoxStrides bs = strides(b, c);
        void *U0 = c.U[0], *U1 = c.U[1], *B0 = c.B[0], *B1 = c.B[1];
        const void* dt = static_cast<char*>(c.clock) + 2 * b->elem;
        CflFinalizeArgs fa{};
        fa.part = c.part;
        fa.nparts = c.cfl_nparts;
        fa.u = U0;
        fa.b = B0;
        fa.nx = fa.ny = fa.nz = n;
        fa.cfl = cfl;
        fa.advance = 1;
        fa.clock = c.clock;
        fa.nsteps = b->nsteps_dev;
        fa.err = b->err_dev;
        fa.bs = bs;
        BTRY(cu(b->ks->cfl_finalize(fa, b->stream)));
        // the side array (classes with c.side): written by the forward fluidx launches
        // and the backward transposes, read by the advectbyzx after them, as in
        // the single-box plain step
        void* const Wf = (c.side && b->ks->fluidx_writes_w(n, n, n, tma_ok(b, n))) ? c.W : nullptr;
        auto Wt = [&](int axis) -> void* {
            return (c.side && b->ks->transpose_writes_w(axis, n, n, n)) ? c.W : nullptr;
        };
        auto F = [&](void* uo, const void* uu, const void* ub, void* part, void* w_out) {
            FluidxArgs a{};
            a.u_out = uo;
            a.uu = uu;
            a.ub = ub;
            a.nx = a.ny = a.nz = n;
            a.use_tma = tma_ok(b, n);
            a.dt_ptr = dt;
            a.cfl_part = part;
            a.err = b->err_dev;
            a.bs = bs;
            a.w_out = w_out;
            b->launches++;
            return cu(b->ks->fluidx(a, b->stream));
        };
        auto A = [&](void* bo, const void* b1, const void* uu, const void* ub, const void* w) {
            AdvectArgs a{};
            a.b_out = bo;
            a.b1_src = b1;
            a.uu = uu;
            a.ub = ub;
            a.nx = a.ny = a.nz = n;
            a.dt_ptr = dt;
            a.err = b->err_dev;
            a.bs = bs;
            a.w = w;
            b->launches++;
            return cu(b->ks->advect(a, b->stream));
        };
        auto T = [&](int axis, void* uo, void* bo, const void* uu, const void* ub, void* w_out) {
            TransposeArgs a{uo, bo, uu, ub, n, n, n, axis};
            a.err = b->err_dev;
            a.bs = bs;
            a.w_out = w_out;
            b->launches++;
            return cu(b->ks->transpose(a, b->stream));
        };
        b->launches++;
        BTRY(F(U1, U0, B0, nullptr, Wf));
        BTRY(A(B1, B0, U1, B0, Wf));
        BTRY(T(1, U0, B0, U1, B1, nullptr));
        BTRY(F(U1, U0, B0, nullptr, Wf));
        BTRY(A(B1, B0, U1, B0, Wf));
        BTRY(T(2, U0, B0, U1, B1, nullptr));
        BTRY(F(U1, U0, B0, nullptr, Wf));
        BTRY(A(B1, B0, U1, B0, Wf));
        BTRY(A(B0, B1, U1, B1, Wf));
        BTRY(F(U0, U1, B0, nullptr, nullptr));
        void* W2 = Wt(2);
        BTRY(T(2, U1, B1, U0, B0, W2));
        BTRY(A(B0, B1, U1, B1, W2));
        BTRY(F(U0, U1, B0, nullptr, nullptr));
        void* W1 = Wt(1);
        BTRY(T(1, U1, B1, U0, B0, W1));
        BTRY(A(B0, B1, U1, B1, W1));
        BTRY(F(U0, U1, B0, c.part, nullptr));  // with the CFL partials of the next step
        c.cfl_nparts = b->ks->fluidx_parts(n, n, n, tma_ok(b, n));
    }
    return enqueue_multi(b, cfl);
}

// One Strang step of the work-list group: the sequence of enqueue_step, each
// operator one launch over every class of the group (largest first), with the
// side array written by the forward fluidx launches and by both backward
// transposes (every transpose kind of the work list writes it).
static int enqueue_multi(mhd_batch* b, double cfl)
{
    std::vector<SizeClass*> g;
    for (auto& c : b->cls)
        if (c.multi)
            g.push_back(&c);
    if (g.empty())
        return MHD_OK;
    std::stable_sort(g.begin(), g.end(), [](const SizeClass* x, const SizeClass* y) {
        return x->cells() * x->boxes.size() > y->cells() * y->boxes.size();
    });
    const int ns = (int)g.size();
    const size_t dt_off = 2 * (size_t)b->elem;
    {
        CflFinalizeArgs fa[kMaxSegs];
        for (int i = 0; i < ns; i++) {
            SizeClass& c = *g[i];
            CflFinalizeArgs x{};
            x.part = c.part;
            x.nparts = c.cfl_nparts;
            x.u = c.U[0];
            x.b = c.B[0];
            x.nx = x.ny = x.nz = c.n;
            x.cfl = cfl;
            x.advance = 1;
            x.clock = c.clock;
            x.nsteps = b->nsteps_dev;
            x.err = b->err_dev;
            x.bs = strides(b, c);
            fa[i] = x;
        }
        b->launches++;
        BTRY(cu(b->ks->finalize_multi(fa, ns, b->stream)));
    }
    // buffer selectors: 0 / 1 = the first / second of each class's ping-pong pair
    auto F = [&](int uo, int uu, int ub, bool part, bool w) {
        FluidxArgs a[kMaxSegs];
        for (int i = 0; i < ns; i++) {
            SizeClass& c = *g[i];
            FluidxArgs x{};
            x.u_out = c.U[uo];
            x.uu = c.U[uu];
            x.ub = c.B[ub];
            x.nx = x.ny = x.nz = c.n;
            x.use_tma = 1;
            x.dt_ptr = static_cast<char*>(c.clock) + dt_off;
            x.cfl_part = part ? c.part : nullptr;
            x.err = b->err_dev;
            x.bs = strides(b, c);
            x.w_out = w ? c.W : nullptr;
            a[i] = x;
        }
        b->launches++;
        return cu(b->ks->fluidx_multi(a, ns, b->stream));
    };
    auto A = [&](int bo, int b1, int uu, int ub) {
        AdvectArgs a[kMaxSegs];
        for (int i = 0; i < ns; i++) {
            SizeClass& c = *g[i];
            AdvectArgs x{};
            x.b_out = c.B[bo];
            x.b1_src = c.B[b1];
            x.uu = c.U[uu];
            x.ub = c.B[ub];
            x.nx = x.ny = x.nz = c.n;
            x.dt_ptr = static_cast<char*>(c.clock) + dt_off;
            x.err = b->err_dev;
            x.bs = strides(b, c);
            x.w = c.W;
            a[i] = x;
        }
        b->launches++;
        return cu(b->ks->advect_multi(a, ns, b->stream));
    };
    auto T = [&](int axis, int uo, int bo, int uu, int ub, bool w) {
        TransposeArgs a[kMaxSegs];
        for (int i = 0; i < ns; i++) {
            SizeClass& c = *g[i];
            TransposeArgs x{c.U[uo], c.B[bo], c.U[uu], c.B[ub], c.n, c.n, c.n, axis};
            x.err = b->err_dev;
            x.bs = strides(b, c);
            x.w_out = w ? c.W : nullptr;
            a[i] = x;
        }
        b->launches++;
        return cu(b->ks->transpose_multi(a, ns, b->stream));
    };
    BTRY(F(1, 0, 0, false, true));
    BTRY(A(1, 0, 1, 0));
    BTRY(T(1, 0, 0, 1, 1, false));
    BTRY(F(1, 0, 0, false, true));
    BTRY(A(1, 0, 1, 0));
    BTRY(T(2, 0, 0, 1, 1, false));
    BTRY(F(1, 0, 0, false, true));
    BTRY(A(1, 0, 1, 0));
    BTRY(A(0, 1, 1, 1));
    BTRY(F(0, 1, 0, false, false));
    BTRY(T(2, 1, 1, 0, 0, true));
    BTRY(A(0, 1, 1, 1));
    BTRY(F(0, 1, 0, false, false));
    BTRY(T(1, 1, 1, 0, 0, true));
    BTRY(A(0, 1, 1, 1));
    BTRY(F(0, 1, 0, true, false));  // with the CFL partials of the next step
    for (SizeClass* c : g)
        c->cfl_nparts = b->ks->multi_fluidx_parts(c->n);
    return MHD_OK;
}

static bool steady(mhd_batch* b)
{
    assign_worklist(b);
    for (auto& c : b->cls)
        if (c.cfl_nparts != fluidx_parts_of(b, c))
            return false;
    return true;
}

extern "C" MHD_API int mhd_batch_step(mhd_batch* b, int nsteps, double cfl)
{
    if (!b || nsteps < 0 || !(cfl > 0))
        return MHD_ERR_ARG;
    for (char l : b->loaded)
        if (!l)
            return MHD_ERR_ARG;
    for (int s = 0; s < nsteps; s++) {
        if (!b->cfl_valid)
            BTRY(cfl_first_pass(b));
        if (!steady(b)) {  // the first step after a standalone calcfl runs uncaptured
            BTRY(enqueue_step(b, cfl));
            continue;
        }
        if (!b->graph || b->gcfl != cfl || b->gtune != tune_generation()) {
            if (b->graph) {
                cudaGraphExecDestroy(b->graph);
                b->graph = nullptr;
            }
            cudaGraph_t g = nullptr;
            BTRY(cu(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal)));
            const long long before = b->launches;
            const int st = enqueue_step(b, cfl);
            const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
            b->glaunches = (int)(b->launches - before);
            b->launches = before;
            if (st != MHD_OK) {
                if (g)
                    cudaGraphDestroy(g);
                return st;
            }
            BTRY(cu(e));
            const cudaError_t ei = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            BTRY(cu(ei));
            b->gcfl = cfl;
            b->gtune = tune_generation();
        }
        BTRY(cu(cudaGraphLaunch(b->graph, b->stream)));
        b->launches += b->glaunches;
    }
    return MHD_OK;
}

extern "C" MHD_API int mhd_batch_sync(mhd_batch* b)
{
    if (!b)
        return MHD_ERR_ARG;
    BTRY(cu(cudaStreamSynchronize(b->stream)));
    int herr = 0;
    BTRY(cu(cudaMemcpy(&herr, b->err_dev, sizeof(int), cudaMemcpyDeviceToHost)));
    if (herr & DEVERR_TIMEOUT)
        return MHD_ERR_TIMEOUT;
    if (herr & DEVERR_NONFINITE)
        return MHD_ERR_NONFINITE;
    return MHD_OK;
}

extern "C" MHD_API void* mhd_batch_stream(mhd_batch* b) { return b ? (void*)b->stream : nullptr; }

extern "C" MHD_API long long mhd_batch_launch_count(mhd_batch* b) { return b ? b->launches : -1; }

extern "C" MHD_API int mhd_batch_classes(mhd_batch* b) { return b ? (int)b->cls.size() : -1; }

extern "C" MHD_API int mhd_batch_set_worklist(mhd_batch* b, int on)
{
    if (!b)
        return MHD_ERR_ARG;
    if (b->worklist != (on != 0)) {
        b->worklist = (on != 0);
        if (b->graph) {  // the step graph holds the other grouping
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
    }
    return MHD_OK;
}

extern "C" MHD_API int mhd_batch_worklist_classes(mhd_batch* b)
{
    if (!b)
        return -1;
    assign_worklist(b);
    int k = 0;
    for (auto& c : b->cls)
        k += c.multi ? 1 : 0;
    return k;
}

extern "C" MHD_API int mhd_batch_tune_edge(mhd_batch* b, int edge, const char* key, int value)
{
    const int k = tune_index(key);
    if (!b || k < 0 || value < -1)
        return MHD_ERR_ARG;
    int hit = 0;
    for (auto& c : b->cls)
        if (c.n == edge) {
            c.knobs[k] = value;
            hit = 1;
        }
    if (!hit)
        return MHD_ERR_ARG;
    if (b->graph) {  // the step graph holds the old launch shapes
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return MHD_OK;
}
