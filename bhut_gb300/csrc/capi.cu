// C ABI of the engine (include/bhut_gb300.h): tree handles, host/device
// pointer staging, and the build / refit / traversal pipelines.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include <utility>
#include "../../include/bhut_gb300.h"
#include "tree.cuh"

namespace bhut {

// ---- error reporting --------------------------------------------------------
static thread_local std::string g_last_error;

void set_error(const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

static std::atomic<long long> g_launches{0};

void note_launches(long long k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

int cuda_status(cudaError_t e, const char* what)
{
    set_error("CUDA error %s (%s) in %s", cudaGetErrorName(e), cudaGetErrorString(e), what);
    return e == cudaErrorMemoryAllocation ? kNoMemory : kCuda;
}

// ---- device buffers -----------------------------------------------------------
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    int ensure(size_t need, cudaStream_t s)
    {
        if (need <= bytes && p) return kOk;
        if (p) {
            BHUT_CUDA(cudaFreeAsync(p, s));
            p = nullptr;
            bytes = 0;
        }
        size_t want = need < 256 ? 256 : need;
        cudaError_t e = cudaMallocAsync(&p, want, s);
        if (e != cudaSuccess) {
            p = nullptr;
            return cuda_status(e, "cudaMallocAsync");
        }
        bytes = want;
        return kOk;
    }
    void release(cudaStream_t s)
    {
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
        bytes = 0;
    }
    template <class T> T* as() const { return (T*)p; }
};

bool is_device_pointer(const void* p)
{
    if (!p) return false;
    cudaPointerAttributes a;
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Copies n bytes from a host or device pointer into a device buffer.
int stage_in(DevBuf& dst, const void* src, size_t bytes, cudaStream_t s)
{
    BHUT_TRY(dst.ensure(bytes, s));
    if (bytes == 0) return kOk;
    BHUT_CUDA(cudaMemcpyAsync(dst.p, src, bytes,
                              is_device_pointer(src) ? cudaMemcpyDeviceToDevice
                                                     : cudaMemcpyHostToDevice, s));
    return kOk;
}

}  // namespace bhut

using namespace bhut;

// A build captured as a CUDA graph, with the buffers and sizes it was
// captured for.
struct BuildGraph {
    static constexpr int kKey = 28;
    cudaGraphExec_t exec = nullptr;
    const void* key[kKey] = {};
    long long launches = 0;
    void reset()
    {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
    }
};

struct bhut_tree {
    int dim = 3;
    int leaf = 32;
    int form = BHUT_FORM_EXACT;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool built = false;
    int64_t n = 0;
    int64_t m = 0;
    TopoTables tt{};
    bool topo_valid = false;
    // particles
    DevBuf pos, mass, keys, perm, sx, sy, sz, sm;
    DevBuf pos_in, mass_in;   // new inputs, checked before they replace pos / mass
    // nodes
    DevBuf cm, size, center, half, lo, hi, first_child, start, count, parent, leaf_list, arrive;
    // scratch
    DevBuf sort_scratch, box_partial, box, counters, err, stats;
    DevBuf frontier;          // bottom-up scratch: one entry per leaf
    DevBuf box_in;            // bounding box of pos_in, computed while staging
    bool box_in_valid = false;
    BuildGraph graphs[2];     // captured builds (see do_build)
    int graph_next = 0;
    bool graph_unsupported = false;
    unsigned long long last_stats[5] = {0, 0, 0, 0, 0};
    // traversal targets
    DevBuf tpos, tkeys, tperm, tx, ty, tz, tbox, out;
    // float-float copies for the fast form
    DevBuf frame, ph, pl, nh, nl, nsize, ndelta, th, tl, quad, nq0, nq1, nhdr;
    bool ff_valid = false;
    bool ff_quad = false;
    int mac = 0;
    int multipole = BHUT_MULTIPOLE_MONO;

    TreeDev dev() const
    {
        TreeDev t;
        t.dim = dim;
        t.leaf_size = leaf;
        t.n = n;
        t.m = m;
        t.sx = sx.as<double>();
        t.sy = sy.as<double>();
        t.sz = sz.as<double>();
        t.sm = sm.as<double>();
        t.perm = perm.as<int32_t>();
        t.cm = cm.as<NodeCM>();
        t.size = size.as<double>();
        t.first_child = first_child.as<int32_t>();
        t.start = start.as<int32_t>();
        t.count = count.as<int32_t>();
        return t;
    }
    NodeOut nodes() const
    {
        return NodeOut{cm.as<NodeCM>(), size.as<double>(), center.as<double>(), half.as<double>(),
                       lo.as<double>(), hi.as<double>()};
    }
};

namespace {

int check_err_word(bhut_tree* t, const char* what)
{
    unsigned e = 0;
    BHUT_CUDA(cudaMemcpyAsync(&e, t->err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, t->stream));
    BHUT_CUDA(cudaStreamSynchronize(t->stream));
    if (e == 0) return kOk;
    BHUT_CUDA(cudaMemsetAsync(t->err.p, 0, sizeof(unsigned), t->stream));
    if (e & kErrNonFinite) {
        set_error("positions must be finite (NaN or Inf found) in %s", what);
        return kInvalid;
    }
    set_error("device error word 0x%x in %s", e, what);
    return kDeviceFlag;
}

// Morton keys + stable sort of `n` AoS points into keys/perm (perm is the
// sort payload, original index).  Uses the handle's scratch.
int sort_points(bhut_tree* t, const double* dpos, const double* dmass, int64_t n, DevBuf& keys,
                DevBuf& perm, DevBuf& box)
{
    cudaStream_t s = t->stream;
    BHUT_TRY(keys.ensure(sizeof(uint64_t) * n, s));
    BHUT_TRY(perm.ensure(sizeof(int32_t) * n, s));
    BHUT_TRY(box.ensure(sizeof(double) * kBoxDoubles, s));
    BHUT_TRY(t->box_partial.ensure(sizeof(double) * kBoxPartialDoubles, s));
    BHUT_TRY(launch_bbox(dpos, dmass, n, t->dim, t->box_partial.as<double>(),
                         t->counters.as<unsigned>(), box.as<double>(), t->err.as<unsigned>(), s));
    BHUT_TRY(launch_morton(dpos, n, t->dim, box.as<double>(), keys.as<uint64_t>(),
                           perm.as<int32_t>(), s));
    BHUT_TRY(t->sort_scratch.ensure(sort_scratch_bytes(n), s));
    BHUT_TRY(radix_sort_pairs(keys.as<uint64_t>(), perm.as<int32_t>(), n, t->dim == 3 ? 63 : 42,
                              t->sort_scratch.p, s));
    return kOk;
}

// Kernels of one build after its buffers exist: Morton keys, radix sort,
// Morton-ordered copies, node moments.  Captured into a CUDA graph by
// do_build (enqueue only: no allocation, no host synchronisation).
int enqueue_build(bhut_tree* t, int64_t n)
{
    cudaStream_t s = t->stream;
    const int dim = t->dim;
    BHUT_TRY(launch_morton(t->pos.as<double>(), n, dim, t->box.as<double>(),
                           t->keys.as<uint64_t>(), t->perm.as<int32_t>(), s));
    BHUT_TRY(radix_sort_pairs(t->keys.as<uint64_t>(), t->perm.as<int32_t>(), n,
                              dim == 3 ? 63 : 42, t->sort_scratch.p, s));
    BHUT_TRY(launch_gather(t->pos.as<double>(), t->mass.as<double>(), t->perm.as<int32_t>(), n, dim,
                           t->sx.as<double>(), t->sy.as<double>(), t->sz.as<double>(),
                           t->sm.as<double>(), s));
    BHUT_TRY(launch_bottom_up(t->dev(), t->leaf_list.as<int32_t>(), t->tt.num_leaves,
                              t->first_child.as<int32_t>(), t->start.as<int32_t>(),
                              t->count.as<int32_t>(), t->parent.as<int32_t>(),
                              t->arrive.as<unsigned>(), t->nodes(), false, nullptr, nullptr,
                              t->frontier.as<int32_t>(), t->counters.as<unsigned>() + 6,
                              t->err.as<unsigned>(), s));
    return kOk;
}

// The buffers a build graph reads and writes, plus its sizes: a captured
// graph is replayed only while all of them are unchanged.
void build_graph_key(const bhut_tree* t, int64_t n, const void** key)
{
    const DevBuf* bufs[] = {&t->pos, &t->mass, &t->box, &t->keys, &t->perm, &t->sort_scratch,
                            &t->sx, &t->sy, &t->sz, &t->sm, &t->cm, &t->size, &t->center,
                            &t->half, &t->lo, &t->hi, &t->arrive, &t->first_child, &t->start,
                            &t->count, &t->parent, &t->leaf_list, &t->err, &t->counters,
                            &t->frontier};
    int k = 0;
    for (const DevBuf* b : bufs) key[k++] = b->p;
    key[k++] = (const void*)(intptr_t)n;
    key[k++] = (const void*)(intptr_t)t->tt.num_leaves;
    key[k++] = (const void*)t->stream;
}

int do_build(bhut_tree* t, int64_t n)
{
    cudaStream_t s = t->stream;
    const int dim = t->dim;
    if (n != t->tt.n || !t->topo_valid) {
        BHUT_TRY(make_topo_tables(n, t->leaf, &t->tt));
        t->topo_valid = false;
    }
    t->n = n;
    t->m = t->tt.num_nodes;
    const int64_t m = t->m;
    // every buffer first (no allocation may happen inside a captured graph)
    BHUT_TRY(t->keys.ensure(sizeof(uint64_t) * n, s));
    BHUT_TRY(t->perm.ensure(sizeof(int32_t) * n, s));
    BHUT_TRY(t->box.ensure(sizeof(double) * kBoxDoubles, s));
    BHUT_TRY(t->box_partial.ensure(sizeof(double) * kBoxPartialDoubles, s));
    BHUT_TRY(t->sort_scratch.ensure(sort_scratch_bytes(n), s));
    for (DevBuf* b : {&t->sx, &t->sy, &t->sz, &t->sm}) BHUT_TRY(b->ensure(sizeof(double) * n, s));
    BHUT_TRY(t->cm.ensure(sizeof(NodeCM) * m, s));
    for (DevBuf* b : {&t->size, &t->half}) BHUT_TRY(b->ensure(sizeof(double) * m, s));
    BHUT_TRY(t->center.ensure(sizeof(double) * m * dim, s));
    BHUT_TRY(t->lo.ensure(sizeof(double) * m * 3, s));
    BHUT_TRY(t->hi.ensure(sizeof(double) * m * 3, s));
    BHUT_TRY(t->arrive.ensure(sizeof(unsigned) * m, s));
    BHUT_TRY(t->frontier.ensure(sizeof(int32_t) * m, s));
    if (!t->topo_valid) {
        for (DevBuf* b : {&t->first_child, &t->start, &t->count, &t->parent})
            BHUT_TRY(b->ensure(sizeof(int32_t) * m, s));
        BHUT_TRY(t->leaf_list.ensure(sizeof(int32_t) * t->tt.num_leaves, s));
        BHUT_TRY(launch_topology(t->tt, t->first_child.as<int32_t>(), t->start.as<int32_t>(),
                                 t->count.as<int32_t>(), t->parent.as<int32_t>(),
                                 t->leaf_list.as<int32_t>(), t->counters.as<unsigned>() + 1,
                                 t->err.as<unsigned>(), s));
        BHUT_TRY(t->tkeys.ensure(sizeof(uint64_t) * t->tt.num_leaves, s));
        BHUT_TRY(order_leaves(t->leaf_list.as<int32_t>(), t->tt.num_leaves,
                              t->start.as<int32_t>(), t->tkeys.as<uint64_t>(),
                              t->sort_scratch.p, s));
        t->topo_valid = true;
    }
    // the box of these positions was computed while they were staged
    if (t->box_in_valid) {
        std::swap(t->box, t->box_in);
    } else {
        BHUT_TRY(launch_bbox(t->pos.as<double>(), t->mass.as<double>(), n, dim,
                             t->box_partial.as<double>(), t->counters.as<unsigned>(),
                             t->box.as<double>(), t->err.as<unsigned>(), s));
    }
    t->box_in_valid = false;
    // replay a captured graph of this exact buffer set; capture one when the
    // same buffer set comes back (a handle built once, as by
    // accelerations(), launches its kernels directly); two are kept: staging
    // alternates between two position buffers
    const void* key[BuildGraph::kKey];
    build_graph_key(t, n, key);
    BuildGraph* g = nullptr;
    BuildGraph* seen = nullptr;
    for (BuildGraph& c : t->graphs) {
        if (std::equal(key, key + BuildGraph::kKey, c.key)) {
            if (c.exec) g = &c;
            else seen = &c;
        }
    }
    if (!g && (!seen || t->graph_unsupported)) {
        BuildGraph& slot = seen ? *seen : t->graphs[t->graph_next];
        if (!seen) t->graph_next ^= 1;
        slot.reset();
        std::copy(key, key + BuildGraph::kKey, slot.key);   // remembered, not captured
        BHUT_TRY(enqueue_build(t, n));
    } else if (!g) {
        BuildGraph& slot = *seen;
        const long long l0 = bhut_launch_count();
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            int st = enqueue_build(t, n);
            e = cudaStreamEndCapture(s, &graph);
            if (st != kOk) {
                if (e == cudaSuccess && graph) cudaGraphDestroy(graph);
                return st;
            }
            if (e == cudaSuccess) {
                e = cudaGraphInstantiate(&slot.exec, graph, 0);
                cudaGraphDestroy(graph);
            }
        }
        if (e == cudaSuccess) {
            slot.launches = bhut_launch_count() - l0;
            g = &slot;
        } else {
            // a stream that cannot be captured (e.g. the legacy default
            // stream): launch the kernels directly from now on
            cudaGetLastError();
            slot.reset();
            t->graph_unsupported = true;
            BHUT_TRY(enqueue_build(t, n));
        }
    } else {
        note_launches(g->launches);
    }
    if (g) BHUT_CUDA(cudaGraphLaunch(g->exec, s));
    t->ff_valid = false;
    int st = check_err_word(t, "build");
    if (st != kOk) {
        t->built = false;
        return st;
    }
    t->built = true;
    return kOk;
}

int load_particles(bhut_tree* t, const double* positions, const double* masses, int64_t n)
{
    if (n <= 0) {
        set_error("Cannot build tree with zero particles");
        return kInvalid;
    }
    if (n > 0x7fffffffLL) {
        set_error("at most 2^31-1 particles are supported");
        return kInvalid;
    }
    if (!positions) { set_error("positions is NULL"); return kInvalid; }
    if (!masses && (n != t->n || !t->mass.p)) {
        set_error("masses are required when the particle count changes");
        return kInvalid;
    }
    // stage and check first: a rejected input leaves the built tree intact.
    // One kernel copies device inputs into the staging buffers, checks them
    // for NaN/Inf and computes their bounding box (host inputs are copied
    // in first and then only read).
    cudaStream_t s = t->stream;
    const size_t pbytes = sizeof(double) * n * t->dim;
    BHUT_TRY(t->pos_in.ensure(pbytes, s));
    const double* psrc = t->pos_in.as<double>();
    double* pcopy = nullptr;
    if (is_device_pointer(positions)) {
        psrc = positions;
        pcopy = t->pos_in.as<double>();
    } else {
        BHUT_CUDA(cudaMemcpyAsync(t->pos_in.p, positions, pbytes, cudaMemcpyHostToDevice, s));
    }
    const double* msrc = t->mass.as<double>();   // masses=None: the current masses
    double* mcopy = nullptr;
    if (masses) {
        BHUT_TRY(t->mass_in.ensure(sizeof(double) * n, s));
        msrc = t->mass_in.as<double>();
        if (is_device_pointer(masses)) {
            msrc = masses;
            mcopy = t->mass_in.as<double>();
        } else {
            BHUT_CUDA(cudaMemcpyAsync(t->mass_in.p, masses, sizeof(double) * n,
                                      cudaMemcpyHostToDevice, s));
        }
    }
    unsigned* flag = t->counters.as<unsigned>() + 4;
    BHUT_CUDA(cudaMemsetAsync(flag, 0, sizeof(unsigned), s));
    BHUT_TRY(t->box_in.ensure(sizeof(double) * kBoxDoubles, s));
    BHUT_TRY(t->box_partial.ensure(sizeof(double) * kBoxPartialDoubles, s));
    BHUT_TRY(launch_stage_bbox(psrc, msrc, n, t->dim, pcopy, mcopy, t->box_partial.as<double>(),
                               t->counters.as<unsigned>(), t->box_in.as<double>(), flag, s));
    unsigned bad = 0;
    BHUT_CUDA(cudaMemcpyAsync(&bad, flag, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    BHUT_CUDA(cudaStreamSynchronize(s));
    if (bad) {
        set_error("positions must be finite (NaN or Inf found)");
        return kInvalid;
    }
    std::swap(t->pos, t->pos_in);
    if (masses) std::swap(t->mass, t->mass_in);
    t->box_in_valid = true;
    return kOk;
}

// Writes a device result either straight into a device out pointer or via a
// device buffer and a copy to host memory.
struct OutTarget {
    double* dev;
    double* host;
};

int out_target(bhut_tree* t, double* out, size_t bytes, OutTarget* o)
{
    if (is_device_pointer(out)) {
        o->dev = out;
        o->host = nullptr;
        return kOk;
    }
    BHUT_TRY(t->out.ensure(bytes, t->stream));
    o->dev = t->out.as<double>();
    o->host = out;
    return kOk;
}

int finish_out(bhut_tree* t, const OutTarget& o, size_t bytes, const char* what)
{
    if (o.host && bytes)
        BHUT_CUDA(cudaMemcpyAsync(o.host, o.dev, bytes, cudaMemcpyDeviceToHost, t->stream));
    return check_err_word(t, what);
}

// Float-float copies of particles and nodes for the fast form (built once
// per build/refit, on first use).
int prepare_fast(bhut_tree* t)
{
    const bool want_quad = t->multipole == BHUT_MULTIPOLE_QUAD && t->form == BHUT_FORM_FP32;
    if (t->ff_valid && t->ff_quad == want_quad) return kOk;
    cudaStream_t s = t->stream;
    BHUT_TRY(t->frame.ensure(sizeof(FastFrame), s));
    BHUT_TRY(t->ph.ensure(sizeof(float4) * t->n, s));
    BHUT_TRY(t->pl.ensure(sizeof(float4) * t->n, s));
    BHUT_TRY(t->nh.ensure(sizeof(float4) * t->m, s));
    BHUT_TRY(t->nl.ensure(sizeof(float4) * t->m, s));
    BHUT_TRY(t->nsize.ensure(sizeof(float) * t->m, s));
    BHUT_TRY(t->ndelta.ensure(sizeof(float) * t->m, s));
    BHUT_TRY(t->nhdr.ensure(sizeof(int4) * t->m, s));
    const bool quad = t->multipole == BHUT_MULTIPOLE_QUAD && t->form == BHUT_FORM_FP32;
    if (quad) {
        BHUT_TRY(t->quad.ensure(sizeof(double) * 6 * t->m, s));
        BHUT_TRY(t->nq0.ensure(sizeof(float4) * t->m, s));
        BHUT_TRY(t->nq1.ensure(sizeof(float2) * t->m, s));
        BHUT_TRY(launch_quadrupoles(t->dev(), t->leaf_list.as<int32_t>(), t->tt.num_leaves,
                                    t->first_child.as<int32_t>(), t->start.as<int32_t>(),
                                    t->count.as<int32_t>(), t->parent.as<int32_t>(),
                                    t->arrive.as<unsigned>(), t->quad.as<double>(),
                                    t->frontier.as<int32_t>(), t->counters.as<unsigned>() + 6,
                                    t->err.as<unsigned>(), s));
    }
    BHUT_TRY(launch_fast_prepare(t->box.as<double>(), t->dim, t->frame.as<FastFrame>(), t->dev(),
                                 t->center.as<double>(), t->ph.as<float4>(), t->pl.as<float4>(),
                                 t->nh.as<float4>(), t->nl.as<float4>(), t->nsize.as<float>(),
                                 t->ndelta.as<float>(), quad ? t->quad.as<double>() : nullptr,
                                 t->nq0.as<float4>(), t->nq1.as<float2>(), t->nhdr.as<int4>(),
                                 s));
    t->ff_quad = quad;
    t->ff_valid = true;
    return kOk;
}

FastTree fast_tree(const bhut_tree* t)
{
    return FastTree{t->frame.as<FastFrame>(), t->ph.as<float4>(), t->pl.as<float4>(),
                    t->nh.as<float4>(), t->nl.as<float4>(), t->nsize.as<float>(),
                    t->ndelta.as<float>(), t->ff_quad ? t->nq0.as<float4>() : nullptr,
                    t->ff_quad ? t->nq1.as<float2>() : nullptr, t->nhdr.as<int4>()};
}

// Scale of the fast form's normalised coordinates (the frame's s), read
// back once per traversal to scale the softening.
int frame_scale(bhut_tree* t, double* s_out)
{
    FastFrame f;
    BHUT_CUDA(cudaMemcpyAsync(&f, t->frame.p, sizeof(FastFrame), cudaMemcpyDeviceToHost, t->stream));
    BHUT_CUDA(cudaStreamSynchronize(t->stream));
    *s_out = f.s;
    return kOk;
}

int traverse(bhut_tree* t, const double* tx, const double* ty, const double* tz,
             const int32_t* self_id, const int32_t* out_idx, int64_t nt, double theta, double eps,
             double G, double* out, bool self_targets)
{
    TreeDev d = t->dev();
    BHUT_TRY(t->stats.ensure(sizeof(unsigned long long) * 8, t->stream));
    BHUT_CUDA(cudaMemsetAsync(t->stats.p, 0, sizeof(unsigned long long) * 8, t->stream));
    unsigned long long* st = t->stats.as<unsigned long long>();
    switch (t->form) {
    case BHUT_FORM_FAST:
    case BHUT_FORM_FP32: {
        BHUT_TRY(prepare_fast(t));
        double sc = 1.0;
        BHUT_TRY(frame_scale(t, &sc));
        const float4* th = nullptr;
        const float4* tl = nullptr;
        if (!self_targets) {
            BHUT_TRY(t->th.ensure(sizeof(float4) * nt, t->stream));
            BHUT_TRY(t->tl.ensure(sizeof(float4) * nt, t->stream));
            BHUT_TRY(launch_fast_targets(tx, ty, tz, nt, t->dim, t->frame.as<FastFrame>(),
                                         t->th.as<float4>(), t->tl.as<float4>(), t->stream));
            th = t->th.as<float4>();
            tl = t->tl.as<float4>();
        }
        const double es = eps * sc;
        BHUT_TRY(launch_traverse_fast(d, fast_tree(t), th, tl, tx, ty, tz, self_id, out_idx, nt,
                                      theta, eps, G, es * es, out, t->err.as<unsigned>(), st,
                                      t->stream, t->form == BHUT_FORM_FP32,
                                      t->form == BHUT_FORM_FP32 ? t->mac : 0));
        break;
    }
    case BHUT_FORM_EXACT:
    default:
        BHUT_TRY(launch_traverse_exact(d, tx, ty, tz, self_id, out_idx, nt, theta, eps, G, out,
                                       t->err.as<unsigned>(), st, t->stream));
    }
    BHUT_CUDA(cudaMemcpyAsync(t->last_stats, st, sizeof(unsigned long long) * 5,
                              cudaMemcpyDeviceToHost, t->stream));
    return kOk;
}

}  // namespace

extern "C" {

const char* bhut_version(void) { return "bhut_gb300 0.1.0 (sm_103a)"; }

int bhut_last_error(char* buf, size_t len)
{
    if (buf && len) {
        size_t k = g_last_error.size() < len - 1 ? g_last_error.size() : len - 1;
        memcpy(buf, g_last_error.data(), k);
        buf[k] = 0;
    }
    return (int)g_last_error.size();
}

int bhut_tree_create(int dim, int leaf_size, void* stream, bhut_tree** out)
{
    if (!out) { set_error("out is NULL"); return kInvalid; }
    *out = nullptr;
    if (dim != 2 && dim != 3) { set_error("dim must be 2 or 3, got %d", dim); return kInvalid; }
    if (leaf_size <= 0) { set_error("leaf_size must be positive, got %d", leaf_size); return kInvalid; }
    bhut_tree* t = new bhut_tree();
    t->dim = dim;
    t->leaf = leaf_size;
    if (stream) {
        t->stream = (cudaStream_t)stream;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete t; return cuda_status(e, "cudaStreamCreate"); }
        t->own_stream = true;
    }
    int st = t->counters.ensure(sizeof(unsigned) * 8, t->stream);
    if (st == kOk) st = t->err.ensure(sizeof(unsigned), t->stream);
    if (st == kOk) {
        cudaError_t e = cudaMemsetAsync(t->counters.p, 0, sizeof(unsigned) * 8, t->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(t->err.p, 0, sizeof(unsigned), t->stream);
        if (e != cudaSuccess) st = cuda_status(e, "cudaMemsetAsync");
    }
    if (st != kOk) { bhut_tree_destroy(t); return st; }
    *out = t;
    return kOk;
}

int bhut_tree_build(bhut_tree* t, const double* positions, const double* masses, int64_t n)
{
    if (!t) { set_error("tree is NULL"); return kInvalid; }
    if (!masses) { set_error("masses is NULL"); return kInvalid; }
    BHUT_TRY(load_particles(t, positions, masses, n));   // rejected input: tree unchanged
    t->built = false;
    return do_build(t, n);
}

int bhut_tree_rebuild(bhut_tree* t, const double* positions, const double* masses, int64_t n)
{
    if (!t) { set_error("tree is NULL"); return kInvalid; }
    BHUT_TRY(load_particles(t, positions, masses, n));
    t->built = false;
    return do_build(t, n);
}

int bhut_tree_refit(bhut_tree* t, const double* positions, const double* masses, int64_t n,
                    int* rebuilt)
{
    if (!t) { set_error("tree is NULL"); return kInvalid; }
    if (rebuilt) *rebuilt = 0;
    if (!t->built) {
        set_error("Tree must be built before refitting. Call build() first.");
        return kNotBuilt;
    }
    if (n != t->n) {   // should_refit_vs_rebuild: different particle count
        if (rebuilt) *rebuilt = 1;
        return bhut_tree_rebuild(t, positions, masses, n);
    }
    cudaStream_t s = t->stream;
    BHUT_TRY(load_particles(t, positions, masses, n));
    unsigned* flag = t->counters.as<unsigned>() + 2;
    BHUT_CUDA(cudaMemsetAsync(flag, 0, sizeof(unsigned), s));
    BHUT_TRY(launch_outside_root(t->pos.as<double>(), n, t->dim, t->center.as<double>(),
                                 t->half.as<double>(), flag, s));
    unsigned outside = 0;
    BHUT_CUDA(cudaMemcpyAsync(&outside, flag, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    BHUT_CUDA(cudaStreamSynchronize(s));
    if (outside) {
        if (rebuilt) *rebuilt = 1;
        t->built = false;
        return do_build(t, n);
    }
    // refit_tree: new sorted SoA through the frozen perm, then bottom-up
    BHUT_TRY(launch_gather(t->pos.as<double>(), t->mass.as<double>(), t->perm.as<int32_t>(), n,
                           t->dim, t->sx.as<double>(), t->sy.as<double>(), t->sz.as<double>(),
                           t->sm.as<double>(), s));
    BHUT_TRY(launch_bottom_up(t->dev(), t->leaf_list.as<int32_t>(), t->tt.num_leaves,
                              t->first_child.as<int32_t>(), t->start.as<int32_t>(),
                              t->count.as<int32_t>(), t->parent.as<int32_t>(),
                              t->arrive.as<unsigned>(), t->nodes(), true, t->pos.as<double>(),
                              t->mass.as<double>(), t->frontier.as<int32_t>(),
                              t->counters.as<unsigned>() + 6, t->err.as<unsigned>(), s));
    t->ff_valid = false;
    return check_err_word(t, "refit");
}

int bhut_tree_refit_only(bhut_tree* t, const double* positions, const double* masses, int64_t n)
{
    if (!t) { set_error("tree is NULL"); return kInvalid; }
    if (!t->built) {
        set_error("Tree must be built before refitting. Call build() first.");
        return kNotBuilt;
    }
    if (n != t->n) {
        set_error("new_positions has %lld particles but tree was built with %lld particles",
                  (long long)n, (long long)t->n);
        return kInvalid;
    }
    cudaStream_t s = t->stream;
    BHUT_TRY(load_particles(t, positions, masses, n));
    BHUT_TRY(launch_gather(t->pos.as<double>(), t->mass.as<double>(), t->perm.as<int32_t>(), n,
                           t->dim, t->sx.as<double>(), t->sy.as<double>(), t->sz.as<double>(),
                           t->sm.as<double>(), s));
    BHUT_TRY(launch_bottom_up(t->dev(), t->leaf_list.as<int32_t>(), t->tt.num_leaves,
                              t->first_child.as<int32_t>(), t->start.as<int32_t>(),
                              t->count.as<int32_t>(), t->parent.as<int32_t>(),
                              t->arrive.as<unsigned>(), t->nodes(), true, t->pos.as<double>(),
                              t->mass.as<double>(), t->frontier.as<int32_t>(),
                              t->counters.as<unsigned>() + 6, t->err.as<unsigned>(), s));
    t->ff_valid = false;
    return check_err_word(t, "refit");
}

int bhut_tree_set_form(bhut_tree* t, int form)
{
    if (!t) { set_error("tree is NULL"); return kInvalid; }
    if (form != BHUT_FORM_EXACT && form != BHUT_FORM_FAST && form != BHUT_FORM_FP32) {
        set_error("traversal form %d is not available in this build", form);
        return kInvalid;
    }
    t->form = form;
    return kOk;
}

int bhut_tree_set_multipole(bhut_tree* t, int multipole)
{
    if (!t) { set_error("tree is NULL"); return kInvalid; }
    if (multipole != BHUT_MULTIPOLE_MONO && multipole != BHUT_MULTIPOLE_QUAD) {
        set_error("unknown multipole order %d", multipole);
        return kInvalid;
    }
    t->multipole = multipole;
    return kOk;
}

int bhut_tree_set_criterion(bhut_tree* t, int criterion)
{
    if (!t) { set_error("tree is NULL"); return kInvalid; }
    if (criterion != BHUT_MAC_BH && criterion != BHUT_MAC_OFFSET) {
        set_error("unknown opening criterion %d", criterion);
        return kInvalid;
    }
    t->mac = criterion;
    return kOk;
}

int bhut_tree_accel_self(bhut_tree* t, double theta, double softening, double G, double* out)
{
    if (!t) { set_error("tree is NULL"); return kInvalid; }
    if (!t->built) { set_error("Tree must be built before evaluating accelerations"); return kNotBuilt; }
    if (!out) { set_error("out is NULL"); return kInvalid; }
    if (!(theta >= 0)) { set_error("theta must be non-negative, got %g", theta); return kInvalid; }
    if (!(softening >= 0)) { set_error("softening must be non-negative, got %g", softening); return kInvalid; }
    size_t bytes = sizeof(double) * t->n * t->dim;
    OutTarget o;
    BHUT_TRY(out_target(t, out, bytes, &o));
    BHUT_TRY(traverse(t, t->sx.as<double>(), t->sy.as<double>(), t->sz.as<double>(),
                      t->perm.as<int32_t>(), t->perm.as<int32_t>(), t->n, theta, softening, G,
                      o.dev, true));
    return finish_out(t, o, bytes, "accelerations");
}

int bhut_tree_accel_targets(bhut_tree* t, const double* targets, int64_t mt, double theta,
                            double softening, double G, double* out)
{
    if (!t) { set_error("tree is NULL"); return kInvalid; }
    if (!t->built) { set_error("Tree must be built before evaluating accelerations"); return kNotBuilt; }
    if (mt < 0 || (mt > 0 && (!targets || !out))) { set_error("invalid targets"); return kInvalid; }
    if (!(theta >= 0)) { set_error("theta must be non-negative, got %g", theta); return kInvalid; }
    if (!(softening >= 0)) { set_error("softening must be non-negative, got %g", softening); return kInvalid; }
    if (mt == 0) return kOk;
    if (mt > 0x7fffffffLL) { set_error("at most 2^31-1 targets are supported"); return kInvalid; }
    cudaStream_t s = t->stream;
    const int dim = t->dim;
    size_t bytes = sizeof(double) * mt * dim;
    BHUT_TRY(stage_in(t->tpos, targets, bytes, s));
    // Morton-order the targets (their own box) so each warp's 32 targets are
    // close together; results are scattered back to input order.
    BHUT_TRY(sort_points(t, t->tpos.as<double>(), nullptr, mt, t->tkeys, t->tperm, t->tbox));
    for (DevBuf* b : {&t->tx, &t->ty, &t->tz}) BHUT_TRY(b->ensure(sizeof(double) * mt, s));
    BHUT_TRY(launch_gather(t->tpos.as<double>(), nullptr, t->tperm.as<int32_t>(), mt, dim,
                           t->tx.as<double>(), t->ty.as<double>(), t->tz.as<double>(), nullptr, s));
    int st = check_err_word(t, "targets");
    if (st != kOk) return st;
    OutTarget o;
    BHUT_TRY(out_target(t, out, bytes, &o));
    BHUT_TRY(traverse(t, t->tx.as<double>(), t->ty.as<double>(), t->tz.as<double>(), nullptr,
                      t->tperm.as<int32_t>(), mt, theta, softening, G, o.dev, false));
    return finish_out(t, o, bytes, "accelerations at targets");
}

int bhut_tree_stats(const bhut_tree* t, int64_t* p2p, int64_t* m2p, int64_t* visits)
{
    if (!t) { set_error("tree is NULL"); return kInvalid; }
    if (p2p) *p2p = (int64_t)t->last_stats[0];
    if (m2p) *m2p = (int64_t)t->last_stats[1];
    if (visits) *visits = (int64_t)t->last_stats[2];
    return kOk;
}

int bhut_tree_fallbacks(const bhut_tree* t, int64_t* exact_decisions, int64_t* fp64_pairs)
{
    if (!t) { set_error("tree is NULL"); return kInvalid; }
    if (exact_decisions) *exact_decisions = (int64_t)t->last_stats[3];
    if (fp64_pairs) *fp64_pairs = (int64_t)t->last_stats[4];
    return kOk;
}

long long bhut_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

int bhut_tree_info(const bhut_tree* t, int64_t* n, int64_t* num_nodes, int* dim, int* leaf_size)
{
    if (!t) { set_error("tree is NULL"); return kInvalid; }
    if (n) *n = t->built ? t->n : 0;
    if (num_nodes) *num_nodes = t->built ? t->m : 0;
    if (dim) *dim = t->dim;
    if (leaf_size) *leaf_size = t->leaf;
    return kOk;
}

int bhut_tree_export(const bhut_tree* t, double* center, double* half_size, double* mass,
                     double* com, int64_t* first_child, int64_t* child_count, int64_t* start,
                     int64_t* count, uint8_t* is_leaf, int64_t* perm)
{
    if (!t) { set_error("tree is NULL"); return kInvalid; }
    if (!t->built) { set_error("Tree not built. Call build() first."); return kNotBuilt; }
    const int64_t m = t->m, n = t->n;
    const int dim = t->dim;
    cudaStream_t s = t->stream;
    NodeCM* cm = new NodeCM[m];
    int32_t* fc = new int32_t[m];
    int32_t* st = new int32_t[m];
    int32_t* ct = new int32_t[m];
    int32_t* pm = new int32_t[n];
    int rc = kOk;
    cudaError_t e = cudaMemcpyAsync(cm, t->cm.p, sizeof(NodeCM) * m, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fc, t->first_child.p, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(st, t->start.p, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ct, t->count.p, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(pm, t->perm.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && center) e = cudaMemcpyAsync(center, t->center.p, sizeof(double) * m * dim, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && half_size) e = cudaMemcpyAsync(half_size, t->half.p, sizeof(double) * m, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        rc = cuda_status(e, "export");
    } else {
        for (int64_t k = 0; k < m; k++) {
            if (mass) mass[k] = cm[k].w;
            if (com) {
                com[k * dim] = cm[k].x;
                com[k * dim + 1] = cm[k].y;
                if (dim == 3) com[k * dim + 2] = cm[k].z;
            }
            if (first_child) first_child[k] = fc[k];
            if (child_count) child_count[k] = fc[k] < 0 ? 0 : 2;
            if (start) start[k] = st[k];
            if (count) count[k] = ct[k];
            if (is_leaf) is_leaf[k] = fc[k] < 0 ? 1 : 0;
        }
        if (perm) for (int64_t i = 0; i < n; i++) perm[i] = pm[i];
    }
    delete[] cm; delete[] fc; delete[] st; delete[] ct; delete[] pm;
    return rc;
}

void bhut_tree_destroy(bhut_tree* t)
{
    if (!t) return;
    cudaStream_t s = t->stream;
    DevBuf* all[] = {&t->pos, &t->mass, &t->keys, &t->perm, &t->sx, &t->sy, &t->sz, &t->sm,
                     &t->cm, &t->size, &t->center, &t->half, &t->lo, &t->hi, &t->first_child,
                     &t->start, &t->count, &t->parent, &t->leaf_list, &t->arrive,
                     &t->sort_scratch, &t->box_partial, &t->box, &t->counters, &t->err, &t->stats,
                     &t->tpos, &t->tkeys, &t->tperm, &t->tx, &t->ty, &t->tz, &t->tbox, &t->out,
                     &t->frame, &t->ph, &t->pl, &t->nh, &t->nl, &t->nsize, &t->ndelta, &t->th,
                     &t->tl, &t->quad, &t->nq0, &t->nq1, &t->nhdr, &t->pos_in, &t->mass_in,
                     &t->box_in, &t->frontier};
    for (DevBuf* b : all) b->release(s);
    cudaStreamSynchronize(s);
    for (BuildGraph& g : t->graphs) g.reset();
    if (t->own_stream) cudaStreamDestroy(s);
    delete t;
}

int bhut_morton_keys(const double* positions, int64_t n, int dim, uint64_t* keys, void* stream)
{
    if (dim != 2 && dim != 3) { set_error("dim must be 2 or 3, got %d", dim); return kInvalid; }
    if (n <= 0) { set_error("points array cannot be empty"); return kInvalid; }
    bhut_tree* t = nullptr;
    BHUT_TRY(bhut_tree_create(dim, 1, stream, &t));
    int rc = stage_in(t->pos, positions, sizeof(double) * n * dim, t->stream);
    if (rc == kOk) rc = t->box.ensure(sizeof(double) * kBoxDoubles, t->stream);
    if (rc == kOk) rc = t->box_partial.ensure(sizeof(double) * kBoxPartialDoubles, t->stream);
    if (rc == kOk) rc = t->keys.ensure(sizeof(uint64_t) * n, t->stream);
    if (rc == kOk) rc = launch_bbox(t->pos.as<double>(), nullptr, n, dim, t->box_partial.as<double>(),
                                    t->counters.as<unsigned>(), t->box.as<double>(),
                                    t->err.as<unsigned>(), t->stream);
    if (rc == kOk) rc = launch_morton(t->pos.as<double>(), n, dim, t->box.as<double>(),
                                      t->keys.as<uint64_t>(), nullptr, t->stream);
    if (rc == kOk) {
        cudaError_t e = cudaMemcpyAsync(keys, t->keys.p, sizeof(uint64_t) * n, cudaMemcpyDefault,
                                        t->stream);
        if (e != cudaSuccess) rc = cuda_status(e, "copy keys");
    }
    if (rc == kOk) rc = check_err_word(t, "morton keys");
    bhut_tree_destroy(t);
    return rc;
}

int bhut_morton_argsort(const double* positions, int64_t n, int dim, uint64_t* sorted_keys,
                        int64_t* perm, void* stream)
{
    if (dim != 2 && dim != 3) { set_error("dim must be 2 or 3, got %d", dim); return kInvalid; }
    if (n <= 0) { set_error("points array cannot be empty"); return kInvalid; }
    bhut_tree* t = nullptr;
    BHUT_TRY(bhut_tree_create(dim, 1, stream, &t));
    int rc = stage_in(t->pos, positions, sizeof(double) * n * dim, t->stream);
    if (rc == kOk) rc = sort_points(t, t->pos.as<double>(), nullptr, n, t->keys, t->perm, t->box);
    int32_t* p32 = nullptr;
    if (rc == kOk && sorted_keys) {
        cudaError_t e = cudaMemcpyAsync(sorted_keys, t->keys.p, sizeof(uint64_t) * n,
                                        cudaMemcpyDefault, t->stream);
        if (e != cudaSuccess) rc = cuda_status(e, "copy keys");
    }
    if (rc == kOk && perm) {
        p32 = new int32_t[n];
        cudaError_t e = cudaMemcpyAsync(p32, t->perm.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost,
                                        t->stream);
        if (e != cudaSuccess) rc = cuda_status(e, "copy perm");
    }
    if (rc == kOk) rc = check_err_word(t, "argsort");
    if (rc == kOk && perm) {
        if (is_device_pointer(perm)) {
            int64_t* tmp = new int64_t[n];
            for (int64_t i = 0; i < n; i++) tmp[i] = p32[i];
            cudaError_t e = cudaMemcpy(perm, tmp, sizeof(int64_t) * n, cudaMemcpyHostToDevice);
            if (e != cudaSuccess) rc = cuda_status(e, "copy perm");
            delete[] tmp;
        } else {
            for (int64_t i = 0; i < n; i++) perm[i] = p32[i];
        }
    }
    delete[] p32;
    bhut_tree_destroy(t);
    return rc;
}

int bhut_direct_accelerations(const double* positions, const double* masses, int64_t n, int dim,
                              const double* targets, int64_t mt, double softening, double G,
                              double* out, void* stream)
{
    if (dim != 2 && dim != 3) { set_error("dim must be 2 or 3, got %d", dim); return kInvalid; }
    if (n <= 0) { set_error("Cannot build tree with zero particles"); return kInvalid; }
    if (!targets && mt != n) { set_error("self accelerations need m == n"); return kInvalid; }
    if (mt <= 0) return kOk;
    bhut_tree* t = nullptr;
    BHUT_TRY(bhut_tree_create(dim, 1, stream, &t));
    cudaStream_t s = t->stream;
    int rc = stage_in(t->pos, positions, sizeof(double) * n * dim, s);
    if (rc == kOk) rc = stage_in(t->mass, masses, sizeof(double) * n, s);
    if (rc == kOk && targets) rc = stage_in(t->tpos, targets, sizeof(double) * mt * dim, s);
    DevBuf self_idx;
    if (rc == kOk && !targets) {
        rc = self_idx.ensure(sizeof(int64_t) * n, s);
        if (rc == kOk) {
            int64_t* h = new int64_t[n];
            for (int64_t i = 0; i < n; i++) h[i] = i;
            cudaError_t e = cudaMemcpyAsync(self_idx.p, h, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) rc = cuda_status(e, "copy index");
            delete[] h;
        }
    }
    OutTarget o{nullptr, nullptr};
    size_t bytes = sizeof(double) * mt * dim;
    if (rc == kOk) rc = out_target(t, out, bytes, &o);
    const int chunks = direct_chunks(n, mt);
    DevBuf partial;
    if (rc == kOk && chunks > 1) rc = partial.ensure(sizeof(double) * chunks * mt * dim, s);
    if (rc == kOk) rc = launch_direct(t->pos.as<double>(), t->mass.as<double>(), n, dim,
                                      targets ? t->tpos.as<double>() : nullptr,
                                      targets ? nullptr : self_idx.as<int64_t>(), mt, softening, G,
                                      o.dev, partial.as<double>(), chunks, s);
    if (rc == kOk) rc = finish_out(t, o, bytes, "direct sum");
    self_idx.release(s);
    partial.release(s);
    bhut_tree_destroy(t);
    return rc;
}

// ---- module-level stages (space/bbox.py, utils/morton.py) -------------------
int bhut_aabb(const double* points, int64_t n, int dim, double* pmin, double* pmax, void* stream)
{
    if (dim < 1 || dim > 3) { set_error("dim must be 1 to 3, got %d", dim); return kInvalid; }
    if (n <= 0) { set_error("points array cannot be empty"); return kInvalid; }
    bhut_tree* t = nullptr;
    BHUT_TRY(bhut_tree_create(dim == 1 ? 2 : dim, 1, stream, &t));
    t->dim = dim;
    cudaStream_t s = t->stream;
    int rc = stage_in(t->pos, points, sizeof(double) * n * dim, s);
    if (rc == kOk) rc = t->box.ensure(sizeof(double) * kBoxDoubles, s);
    if (rc == kOk) rc = t->box_partial.ensure(sizeof(double) * kBoxPartialDoubles, s);
    if (rc == kOk) rc = launch_bbox(t->pos.as<double>(), nullptr, n, dim, t->box_partial.as<double>(),
                                    t->counters.as<unsigned>(), t->box.as<double>(),
                                    t->err.as<unsigned>(), s);
    double box[kBoxDoubles];
    if (rc == kOk) {
        cudaError_t e = cudaMemcpyAsync(box, t->box.p, sizeof(box), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_status(e, "copy box");
    }
    // the non-finite flag of the bbox kernel is not an error here: numpy's
    // min/max propagate NaN (an axis holding one gets NaN bounds) and order
    // infinities like any value
    if (rc == kOk) {
        cudaMemsetAsync(t->err.p, 0, sizeof(unsigned), s);
        for (int d = 0; d < dim; d++) {
            const bool has_nan = box[12 + d] != 0.0;
            pmin[d] = has_nan ? NAN : box[d];
            pmax[d] = has_nan ? NAN : box[3 + d];
        }
    }
    bhut_tree_destroy(t);
    return rc;
}

int bhut_normalize_to_unit(const double* points, int64_t n, int dim, const double* pmin,
                           const double* pmax, double eps, double* out, void* stream)
{
    if (dim < 1 || dim > 3) { set_error("dim must be 1 to 3, got %d", dim); return kInvalid; }
    if (n < 0) { set_error("negative point count"); return kInvalid; }
    if (n == 0) return kOk;
    bhut_tree* t = nullptr;
    BHUT_TRY(bhut_tree_create(dim == 1 ? 2 : dim, 1, stream, &t));
    cudaStream_t s = t->stream;
    DevBuf lim;
    int rc = stage_in(t->pos, points, sizeof(double) * n * dim, s);
    if (rc == kOk) rc = lim.ensure(sizeof(double) * 6, s);
    if (rc == kOk) {
        double h[6];
        for (int d = 0; d < dim; d++) { h[d] = pmin[d]; h[3 + d] = pmax[d]; }
        cudaError_t e = cudaMemcpyAsync(lim.p, h, sizeof(h), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_status(e, "copy limits");
    }
    OutTarget o{nullptr, nullptr};
    const size_t bytes = sizeof(double) * n * dim;
    if (rc == kOk) rc = out_target(t, out, bytes, &o);
    if (rc == kOk) rc = launch_normalize(t->pos.as<double>(), n, dim, lim.as<double>(),
                                         lim.as<double>() + 3, 1.0 - eps, o.dev, s);
    if (rc == kOk) rc = finish_out(t, o, bytes, "normalize_to_unit");
    lim.release(s);
    bhut_tree_destroy(t);
    return rc;
}

namespace {
// Morton codes of points in [0, 1)^dim into the handle's keys buffer.
int unit_codes(bhut_tree* t, const double* points01, int64_t n, int dim, int bits)
{
    cudaStream_t s = t->stream;
    BHUT_TRY(stage_in(t->pos, points01, sizeof(double) * n * dim, s));
    BHUT_TRY(t->keys.ensure(sizeof(uint64_t) * n, s));
    unsigned* bad = t->counters.as<unsigned>() + 3;
    BHUT_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned), s));
    BHUT_TRY(launch_morton_unit(t->pos.as<double>(), n, dim, bits, t->keys.as<uint64_t>(), bad, s));
    unsigned h = 0;
    BHUT_CUDA(cudaMemcpyAsync(&h, bad, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    BHUT_CUDA(cudaStreamSynchronize(s));
    if (h) { set_error("All points must be in range [0, 1)"); return kInvalid; }
    return kOk;
}

int check_unit_args(int64_t n, int dim, int bits)
{
    if (dim != 2 && dim != 3) {
        set_error("points01 must have 2 or 3 dimensions, got %d", dim);
        return kInvalid;
    }
    if (bits < 1 || bits > 62) { set_error("bits must be in 1..62, got %d", bits); return kInvalid; }
    if (n < 0) { set_error("negative point count"); return kInvalid; }
    return kOk;
}
}  // namespace

int bhut_morton_codes_unit(const double* points01, int64_t n, int dim, int bits, uint64_t* codes,
                           void* stream)
{
    BHUT_TRY(check_unit_args(n, dim, bits));
    if (n == 0) return kOk;
    bhut_tree* t = nullptr;
    BHUT_TRY(bhut_tree_create(dim, 1, stream, &t));
    int rc = unit_codes(t, points01, n, dim, bits);
    if (rc == kOk) {
        cudaError_t e = cudaMemcpyAsync(codes, t->keys.p, sizeof(uint64_t) * n, cudaMemcpyDefault,
                                        t->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(t->stream);
        if (e != cudaSuccess) rc = cuda_status(e, "copy codes");
    }
    bhut_tree_destroy(t);
    return rc;
}

int bhut_sort_morton_unit(const double* points01, int64_t n, int dim, int bits,
                          uint64_t* sorted_codes, int64_t* perm, void* stream)
{
    BHUT_TRY(check_unit_args(n, dim, bits));
    if (n == 0) return kOk;
    if (n > 0x7fffffffLL) { set_error("at most 2^31-1 points are supported"); return kInvalid; }
    bhut_tree* t = nullptr;
    BHUT_TRY(bhut_tree_create(dim, 1, stream, &t));
    cudaStream_t s = t->stream;
    int rc = unit_codes(t, points01, n, dim, bits);
    if (rc == kOk) rc = t->perm.ensure(sizeof(int32_t) * n, s);
    if (rc == kOk) rc = t->sort_scratch.ensure(sort_scratch_bytes(n), s);
    if (rc == kOk) rc = launch_iota(t->perm.as<int32_t>(), n, s);
    // the interleave masks keep 21 bits per axis in 3-D, 32 in 2-D
    const int key_bits = dim == 3 ? (3 * bits > 63 ? 63 : 3 * bits) : (2 * bits > 64 ? 64 : 2 * bits);
    if (rc == kOk) rc = radix_sort_pairs(t->keys.as<uint64_t>(), t->perm.as<int32_t>(), n, key_bits,
                                         t->sort_scratch.p, s);
    if (rc == kOk && sorted_codes) {
        cudaError_t e = cudaMemcpyAsync(sorted_codes, t->keys.p, sizeof(uint64_t) * n,
                                        cudaMemcpyDefault, s);
        if (e != cudaSuccess) rc = cuda_status(e, "copy codes");
    }
    if (rc == kOk && perm) {
        DevBuf p64;
        rc = p64.ensure(sizeof(int64_t) * n, s);
        if (rc == kOk) rc = launch_widen_i32(t->perm.as<int32_t>(), n, p64.as<int64_t>(), s);
        if (rc == kOk) {
            cudaError_t e = cudaMemcpyAsync(perm, p64.p, sizeof(int64_t) * n, cudaMemcpyDefault, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) rc = cuda_status(e, "copy perm");
        }
        p64.release(s);
    }
    if (rc == kOk) {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_status(e, "sort_by_morton");
    }
    bhut_tree_destroy(t);
    return rc;
}

int bhut_gather_rows(const void* src, int64_t n, int64_t row_bytes, const int64_t* perm, void* dst,
                     void* stream)
{
    if (n < 0 || row_bytes < 0) { set_error("negative size"); return kInvalid; }
    if (n == 0 || row_bytes == 0) return kOk;
    bhut_tree* t = nullptr;
    BHUT_TRY(bhut_tree_create(3, 1, stream, &t));
    cudaStream_t s = t->stream;
    DevBuf dsrc, dperm, ddst;
    const size_t bytes = (size_t)(n * row_bytes);
    int rc = stage_in(dsrc, src, bytes, s);
    if (rc == kOk) rc = stage_in(dperm, perm, sizeof(int64_t) * n, s);
    if (rc == kOk) rc = ddst.ensure(bytes, s);
    if (rc == kOk) rc = launch_gather_rows(dsrc.p, n, row_bytes, dperm.as<int64_t>(), ddst.p,
                                           t->err.as<unsigned>(), s);
    if (rc == kOk) {
        cudaError_t e = cudaMemcpyAsync(dst, ddst.p, bytes, cudaMemcpyDefault, s);
        if (e != cudaSuccess) rc = cuda_status(e, "copy rows");
    }
    if (rc == kOk) rc = check_err_word(t, "gather (permutation index out of range)");
    for (DevBuf* b : {&dsrc, &dperm, &ddst}) b->release(s);
    bhut_tree_destroy(t);
    return rc;
}

int bhut_should_refit(const double* positions, int64_t n, int dim, const double* root_center,
                      double root_half, int* refit, void* stream)
{
    if (dim != 2 && dim != 3) { set_error("dim must be 2 or 3, got %d", dim); return kInvalid; }
    if (!refit) { set_error("result pointer is NULL"); return kInvalid; }
    *refit = 1;
    if (n <= 0) return kOk;
    bhut_tree* t = nullptr;
    BHUT_TRY(bhut_tree_create(dim, 1, stream, &t));
    cudaStream_t s = t->stream;
    DevBuf root;
    int rc = stage_in(t->pos, positions, sizeof(double) * n * dim, s);
    if (rc == kOk) rc = root.ensure(sizeof(double) * 4, s);
    if (rc == kOk) {
        double h[4] = {0, 0, 0, root_half};
        for (int d = 0; d < dim; d++) h[d] = root_center[d];
        cudaError_t e = cudaMemcpyAsync(root.p, h, sizeof(h), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_status(e, "copy root");
    }
    unsigned* flag = t->counters.as<unsigned>() + 2;
    if (rc == kOk) {
        cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(unsigned), s);
        if (e != cudaSuccess) rc = cuda_status(e, "memset");
    }
    if (rc == kOk) rc = launch_outside_root(t->pos.as<double>(), n, dim, root.as<double>(),
                                            root.as<double>() + 3, flag, s);
    unsigned outside = 0;
    if (rc == kOk) {
        cudaError_t e = cudaMemcpyAsync(&outside, flag, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_status(e, "copy flag");
    }
    if (rc == kOk) *refit = outside ? 0 : 1;
    root.release(s);
    bhut_tree_destroy(t);
    return rc;
}

// ---- TreeData import ---------------------------------------------------------
int bhut_tree_import(bhut_tree* t, const double* positions, const double* masses, int64_t n,
                     const int64_t* first_child, const int64_t* child_count, const int64_t* start,
                     const int64_t* count, const int64_t* perm, const double* center,
                     const double* half_size, const double* mass, const double* com,
                     int64_t num_nodes)
{
    if (!t) { set_error("tree is NULL"); return kInvalid; }
    if (num_nodes <= 0 || num_nodes > 0x7fffffffLL) {
        set_error("invalid node count %lld", (long long)num_nodes);
        return kInvalid;
    }
    if (!masses) { set_error("masses are required"); return kInvalid; }
    t->built = false;
    t->topo_valid = false;                 // the next build recomputes its own topology
    BHUT_TRY(load_particles(t, positions, masses, n));
    cudaStream_t s = t->stream;
    const int dim = t->dim;
    const int64_t m = num_nodes;
    DevBuf fc, cc, st, ct, pm, hf, ms, cmn, cen;
    const size_t mi = sizeof(int64_t) * m, md = sizeof(double) * m;
    int rc = stage_in(fc, first_child, mi, s);
    if (rc == kOk) rc = stage_in(cc, child_count, mi, s);
    if (rc == kOk) rc = stage_in(st, start, mi, s);
    if (rc == kOk) rc = stage_in(ct, count, mi, s);
    if (rc == kOk) rc = stage_in(pm, perm, sizeof(int64_t) * n, s);
    if (rc == kOk) rc = stage_in(hf, half_size, md, s);
    if (rc == kOk) rc = stage_in(ms, mass, md, s);
    if (rc == kOk) rc = stage_in(cmn, com, md * dim, s);
    if (rc == kOk) rc = stage_in(cen, center, md * dim, s);
    for (DevBuf* b : {&t->first_child, &t->start, &t->count, &t->parent, &t->leaf_list,
                      &t->frontier})
        if (rc == kOk) rc = b->ensure(sizeof(int32_t) * m, s);
    if (rc == kOk) rc = t->cm.ensure(sizeof(NodeCM) * m, s);
    for (DevBuf* b : {&t->size, &t->half})
        if (rc == kOk) rc = b->ensure(sizeof(double) * m, s);
    if (rc == kOk) rc = t->center.ensure(sizeof(double) * m * dim, s);
    if (rc == kOk) rc = t->lo.ensure(sizeof(double) * m * 3, s);
    if (rc == kOk) rc = t->hi.ensure(sizeof(double) * m * 3, s);
    if (rc == kOk) rc = t->arrive.ensure(sizeof(unsigned) * m, s);
    if (rc == kOk) rc = t->perm.ensure(sizeof(int32_t) * n, s);
    for (DevBuf* b : {&t->sx, &t->sy, &t->sz, &t->sm})
        if (rc == kOk) rc = b->ensure(sizeof(double) * n, s);
    unsigned* leaves = t->counters.as<unsigned>() + 1;
    if (rc == kOk) rc = launch_import_nodes(
        fc.as<int64_t>(), cc.as<int64_t>(), st.as<int64_t>(), ct.as<int64_t>(), hf.as<double>(),
        ms.as<double>(), cmn.as<double>(), cen.as<double>(), m, n, dim,
        t->first_child.as<int32_t>(), t->start.as<int32_t>(), t->count.as<int32_t>(),
        t->parent.as<int32_t>(), t->cm.as<NodeCM>(), t->size.as<double>(), t->half.as<double>(),
        t->center.as<double>(), t->leaf_list.as<int32_t>(), leaves, t->err.as<unsigned>(), s);
    if (rc == kOk) rc = launch_import_perm(pm.as<int64_t>(), n, t->perm.as<int32_t>(),
                                           t->err.as<unsigned>(), s);
    if (rc == kOk) rc = launch_gather(t->pos.as<double>(), t->mass.as<double>(),
                                      t->perm.as<int32_t>(), n, dim, t->sx.as<double>(),
                                      t->sy.as<double>(), t->sz.as<double>(), t->sm.as<double>(), s);
    // the box of the particles frames the float-float forms
    if (rc == kOk) rc = t->box.ensure(sizeof(double) * kBoxDoubles, s);
    if (rc == kOk) rc = t->box_partial.ensure(sizeof(double) * kBoxPartialDoubles, s);
    if (rc == kOk) rc = launch_bbox(t->pos.as<double>(), t->mass.as<double>(), n, dim,
                                    t->box_partial.as<double>(), t->counters.as<unsigned>(),
                                    t->box.as<double>(), t->err.as<unsigned>(), s);
    unsigned nleaves = 0;
    if (rc == kOk) {
        cudaError_t e = cudaMemcpyAsync(&nleaves, leaves, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) rc = cuda_status(e, "copy leaf count");
    }
    if (rc == kOk) rc = check_err_word(t, "tree import (only binary trees with valid ranges)");
    for (DevBuf* b : {&fc, &cc, &st, &ct, &pm, &hf, &ms, &cmn, &cen}) b->release(s);
    if (rc != kOk) return rc;
    t->n = n;
    t->m = m;
    t->tt = TopoTables{};
    t->tt.n = -1;
    t->tt.leaf_size = t->leaf;
    t->tt.num_nodes = m;
    t->tt.num_leaves = nleaves;
    t->ff_valid = false;
    t->built = true;
    return kOk;
}

int bhut_pool_usage(int64_t* used, int64_t* reserved)
{
    if (!used || !reserved) { set_error("result pointer is NULL"); return kInvalid; }
    int dev = 0;
    BHUT_CUDA(cudaGetDevice(&dev));
    cudaMemPool_t pool;
    BHUT_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
    unsigned long long u = 0, r = 0;   // the attributes are 64-bit counts
    BHUT_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &u));
    BHUT_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &r));
    *used = (int64_t)u;
    *reserved = (int64_t)r;
    return kOk;
}

int bhut_pool_trim(void)
{
    int dev = 0;
    BHUT_CUDA(cudaGetDevice(&dev));
    cudaMemPool_t pool;
    BHUT_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
    BHUT_CUDA(cudaDeviceSynchronize());
    BHUT_CUDA(cudaMemPoolTrimTo(pool, 0));
    return kOk;
}

int bhut_measure_fp32_peak(double* tflops)
{
    if (!tflops) { set_error("result pointer is NULL"); return kInvalid; }
    return measure_fp32_peak(tflops);
}

int bhut_tree_statistics(const double* com, const double* half_size, const double* mass,
                         const int64_t* first_child, const int64_t* child_count,
                         const int64_t* start, const int64_t* count, int64_t num_nodes, int dim,
                         const double* targets, int64_t nt, double theta, void* stream,
                         int64_t* totals)
{
    if (dim != 2 && dim != 3) { set_error("dim must be 2 or 3, got %d", dim); return kInvalid; }
    if (num_nodes <= 0 || !totals) { set_error("empty tree"); return kInvalid; }
    if (nt < 0 || (nt > 0 && !targets)) { set_error("invalid targets"); return kInvalid; }
    bhut_tree* t = nullptr;
    BHUT_TRY(bhut_tree_create(dim, 1, stream, &t));
    cudaStream_t s = t->stream;
    DevBuf d_com, d_half, d_mass, d_fc, d_cc, d_start, d_count, d_tot;
    const size_t md = sizeof(double) * num_nodes, mi = sizeof(int64_t) * num_nodes;
    int rc = stage_in(d_com, com, md * dim, s);
    if (rc == kOk) rc = stage_in(d_half, half_size, md, s);
    if (rc == kOk) rc = stage_in(d_mass, mass, md, s);
    if (rc == kOk) rc = stage_in(d_fc, first_child, mi, s);
    if (rc == kOk) rc = stage_in(d_cc, child_count, mi, s);
    if (rc == kOk) rc = stage_in(d_start, start, mi, s);
    if (rc == kOk) rc = stage_in(d_count, count, mi, s);
    if (rc == kOk && nt > 0) rc = stage_in(t->tpos, targets, sizeof(double) * nt * dim, s);
    if (rc == kOk) rc = d_tot.ensure(sizeof(unsigned long long) * 3, s);
    if (rc == kOk) {
        StatTree st{d_com.as<double>(), d_half.as<double>(), d_mass.as<double>(),
                    d_fc.as<int64_t>(), d_cc.as<int64_t>(), d_start.as<int64_t>(),
                    d_count.as<int64_t>(), num_nodes};
        rc = launch_tree_statistics(st, dim, t->tpos.as<double>(), nt, theta,
                                    d_tot.as<unsigned long long>(), t->err.as<unsigned>(), s);
    }
    unsigned long long h[3] = {0, 0, 0};
    if (rc == kOk) {
        cudaError_t e = cudaMemcpyAsync(h, d_tot.p, sizeof(h), cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) rc = cuda_status(e, "copy totals");
    }
    if (rc == kOk) rc = check_err_word(t, "tree statistics");
    if (rc == kOk)
        for (int k = 0; k < 3; k++) totals[k] = (int64_t)h[k];
    for (DevBuf* b : {&d_com, &d_half, &d_mass, &d_fc, &d_cc, &d_start, &d_count, &d_tot})
        b->release(s);
    bhut_tree_destroy(t);
    return rc;
}

}  // extern "C"
