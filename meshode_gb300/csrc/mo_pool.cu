// Native serving runtime: a pool of deformation requests advanced together.
//
// A request is one run of the reference's rigid_deform loop
// (src/python/rigid_deform.py:25-44): normalise the source by the target's
// transform, build the target's distance field, store the rigidity
// information, run `steps` Adam steps of DistanceFieldLoss + RigidEdgeLoss,
// denormalise (Finalize, rigid_loss_layer.py:42-44).  The pool admits
// requests by HBM bytes, prepares them on side streams (copies, DF build, CSR,
// sliced-ELL records) while the step stream replays a captured CUDA graph of
// S fused-step launches over every active pair, and retires a pair right after
// the group in which its last step ran.  All device memory of a request comes
// from the pool's own stream-ordered memory pool, so admissions and
// retirements never synchronise the device.  One host thread drives a pool.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <memory>
#include <unordered_map>
#include <utility>
#include <vector>

#include "mo_common.cuh"

namespace mo {

struct Req {
    int64_t id = 0;
    MoRequest in{};
    int state = MO_REQ_QUEUED;
    int phase = 0;  // 1: phase A issued, 2: phase B issued, 3: active, 4: retiring
    size_t bytes = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr;
    float* srcV = nullptr;  // normalised source (device copy)
    int32_t* srcF = nullptr;
    float* tarV = nullptr;  // device copies when the inputs are on the host
    int32_t* tarF = nullptr;
    int32_t* bbox = nullptr;
    double* params = nullptr;
    int32_t* status = nullptr;  // [0] DF status, [1] edge status, [2] record count
    float* grid = nullptr;
    int32_t* csr = nullptr;
    int32_t* slice_ptr = nullptr;
    int32_t* sell = nullptr;
    float* pos = nullptr;   // 2 x nv float4 (ping-pong)
    float* rest = nullptr;  // nv float4
    float* m = nullptr;
    float* v = nullptr;
    float* result = nullptr;  // [2][nv][3]: normalised, then denormalised
    // on-demand distance field
    bool lazy = false;
    float* tree = nullptr;       // mo_df_tree_build output
    float* lin = nullptr;        // N^3 voxel values
    uint32_t* dfbits = nullptr;  // cell bits, then packet bits
    MoPair* pair_dev = nullptr;  // one-row pair table for the seeding fill
    int32_t* seedq = nullptr;    // seeding queues (nv cells, 8 nv packets) and their counters
    struct HostSlot* host = nullptr;
    int layout = MO_LAYOUT_CELL;
    int spt = MO_TILE_WARPS;
    int method = MO_DF_AUTO;
    int packet = MO_PACKET_4x4x2;
    float band = 0.0f;
    int nslices = 0;
    int ntiles = 0;
    int t = 0;
    const float* adam_tab = nullptr;
    char error[192] = "";
};

// Pinned words a request's status and loss are copied into.
struct HostSlot {
    int32_t status[4];
    double loss;
    double pad;
    MoPair pair;  // the request's pair row for its seeding fill
};

struct AdamTable {
    double lr;
    int rows;
    float* dev;
};

}  // namespace mo

struct MoPool {
    MoPoolConfig cfg{};
    int device = 0;
    cudaStream_t step = nullptr;
    cudaStream_t io = nullptr;  // result copies
    std::vector<cudaStream_t> builds;
    int next_build = 0;
    cudaMemPool_t mempool = nullptr;
    MoPair* pairs_dev = nullptr;
    MoTile* tiles_dev = nullptr;
    int32_t* ntiles_dev = nullptr;
    float* tile_loss = nullptr;
    double* pair_loss = nullptr;
    unsigned char* staging[2] = {nullptr, nullptr};
    cudaEvent_t staging_ev[2] = {nullptr, nullptr};
    int slot = 0;
    std::vector<int64_t> tiles_key;
    cudaGraphExec_t graph = nullptr;
    int64_t next_id = 1;
    std::unordered_map<int64_t, std::unique_ptr<mo::Req>> reqs;
    std::deque<int64_t> queued;
    std::vector<int64_t> building, active, retiring;
    std::deque<int64_t> completed;
    std::vector<mo::AdamTable> adam_tabs;
    std::vector<mo::HostSlot*> slot_chunks, free_slots;
    bool hold = false;
    bool timing = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> group_events;
    std::vector<double> group_bytes;
    int32_t* dfq = nullptr;        // on-demand cells queued by a step: (pair, cell)
    int32_t* dfpq = nullptr;       // and their new voxel packets: (pair, packet)
    int32_t* dfq_count = nullptr;  // two counters (cells, packets) per launch of a group
    int dfq_cap = 0;
    int64_t* fill_totals = nullptr;  // device: cells written, packets computed
    MoPoolStats stats{};
};

namespace mo {
namespace {

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

#define PCHK(call)                                                  \
    do {                                                            \
        cudaError_t _e = (call);                                    \
        if (_e != cudaSuccess) return ::mo::cuda_status(_e, #call); \
    } while (0)

template <class T>
cudaError_t palloc(MoPool* P, T** p, size_t bytes, cudaStream_t s) {
    return cudaMallocFromPoolAsync(reinterpret_cast<void**>(p), a256(bytes ? bytes : 1), P->mempool, s);
}

template <class T>
void pfree(T*& p, cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
}

void free_state(Req* R, cudaStream_t s) {
    pfree(R->srcV, s); pfree(R->srcF, s); pfree(R->tarV, s); pfree(R->tarF, s);
    pfree(R->bbox, s); pfree(R->params, s); pfree(R->status, s); pfree(R->grid, s);
    pfree(R->csr, s); pfree(R->slice_ptr, s); pfree(R->sell, s); pfree(R->pos, s);
    pfree(R->rest, s); pfree(R->m, s); pfree(R->v, s);
    pfree(R->tree, s); pfree(R->lin, s); pfree(R->dfbits, s); pfree(R->pair_dev, s); pfree(R->seedq, s);
}

// Peak device bytes one request holds from admission to retirement.
size_t estimate(const MoRequest& q, int layout, int method, bool lazy) {
    const int64_t nv = q.nv, nh = 3 * q.nf, N = q.N;
    const size_t glin = (size_t)4 * N * N * N;
    size_t grid = layout == MO_LAYOUT_LINEAR ? glin : mo_grid_bytes((int)N, layout) + glin;
    size_t scratch = mo_df_build_scratch_bytes(q.ntv, q.ntf, (int)N, method);
    if (lazy) {
        grid += mo_df_tree_bytes(q.ntf) + mo_df_lazy_bytes((int)N) + sizeof(MoPair) + 72 * (size_t)nv + 256;
        scratch = mo_df_tree_scratch_bytes(q.ntv, q.ntf);
    }
    const size_t meshes = (size_t)12 * (nv + q.nf + q.ntv + q.ntf);
    const size_t edges = mo_edge_csr_bytes(nv, q.nf, MO_EDGES_FACES);
    const size_t sell = (size_t)4 * (2 * nh + 32 * ((nv + 31) / 32) * 4);
    const size_t state = (size_t)(32 + 16 + 12 + 12 + 24) * nv + 4 * ((nv + 31) / 32 + 1);
    return grid + scratch + meshes + edges + sell + state + (1 << 16);
}

// Device table of (lr/(1-b1^t), sqrt(1-b2^t)) for t = 1..rows, each row
// computed in double like torch.optim.Adam's per-step host arithmetic.  A
// table serves every request with the same lr and at most `rows` steps.
int adam_table(MoPool* P, double lr, int steps, const float** out) {
    for (const AdamTable& a : P->adam_tabs)
        if (a.lr == lr && a.rows >= steps) {
            *out = a.dev;
            return MO_OK;
        }
    int rows = 1024;
    while (rows < steps) rows *= 2;
    std::vector<float> tab(2 * (size_t)rows);
    const double b1 = 0.9, b2 = 0.999;
    for (int t = 1; t <= rows; ++t) {
        const double bc1 = 1.0 - std::pow(b1, (double)t), bc2 = 1.0 - std::pow(b2, (double)t);
        tab[2 * (size_t)(t - 1)] = (float)(lr / bc1);
        tab[2 * (size_t)(t - 1) + 1] = (float)std::sqrt(bc2);
    }
    float* d = nullptr;
    PCHK(cudaMalloc(&d, sizeof(float) * tab.size()));
    PCHK(cudaMemcpy(d, tab.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice));
    P->adam_tabs.push_back({lr, rows, d});
    *out = d;
    return MO_OK;
}

void fail(MoPool* P, Req* R, const char* msg, cudaStream_t s) {
    R->state = MO_REQ_FAILED;
    snprintf(R->error, sizeof(R->error), "%s", msg);
    free_state(R, s);
    P->stats.bytes_in_use -= R->bytes;
    R->bytes = 0;
    P->stats.failed += 1;
    P->completed.push_back(R->id);
}

void fill_pair(const MoPool* P, const Req* R, MoPair* p, int tile0);

// Phase A on a build stream: input copies, target bbox and transform, DF
// build (+ re-layout), source normalisation, CSR, sliced-ELL plan; then the
// status words go to pinned host memory.
int phase_a(MoPool* P, Req* R) {
    const MoRequest& q = R->in;
    cudaStream_t s = R->stream;
    void* sv = reinterpret_cast<void*>(s);
    const int64_t nv = q.nv, nf = q.nf;
    const cudaMemcpyKind kind = q.inputs_on_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    PCHK(palloc(P, &R->srcV, 12 * nv, s));
    PCHK(palloc(P, &R->srcF, 12 * nf, s));
    PCHK(cudaMemcpyAsync(R->srcV, q.srcV, 12 * nv, kind, s));
    if (nf) PCHK(cudaMemcpyAsync(R->srcF, q.srcF, 12 * nf, kind, s));
    const float* tarV = q.tarV;
    const int32_t* tarF = q.tarF;
    if (q.inputs_on_host) {
        PCHK(palloc(P, &R->tarV, 12 * q.ntv, s));
        PCHK(palloc(P, &R->tarF, 12 * q.ntf, s));
        PCHK(cudaMemcpyAsync(R->tarV, q.tarV, 12 * q.ntv, kind, s));
        PCHK(cudaMemcpyAsync(R->tarF, q.tarF, 12 * q.ntf, kind, s));
        tarV = R->tarV;
        tarF = R->tarF;
    }
    PCHK(palloc(P, &R->bbox, 32, s));
    PCHK(palloc(P, &R->params, 32, s));
    PCHK(palloc(P, &R->status, 16, s));
    PCHK(cudaMemsetAsync(R->status, 0, 16, s));
    int rc = mo_bbox(tarV, q.ntv, R->bbox, sv);
    if (!rc) rc = mo_norm_params(R->bbox, R->params, sv);
    if (rc) return rc;
    const int N = q.N;
    if (R->lazy) {
        // the tree now; the grid's cells when the steps reach them
        const size_t sb = mo_df_tree_scratch_bytes(q.ntv, q.ntf);
        void* scratch = nullptr;
        PCHK(palloc(P, &scratch, sb, s));
        PCHK(palloc(P, &R->tree, mo_df_tree_bytes(q.ntf), s));
        rc = mo_df_tree_build(tarV, q.ntv, tarF, q.ntf, R->params, scratch, sb, R->tree, R->status, sv);
        cudaFreeAsync(scratch, s);
        if (rc) return rc;
        PCHK(palloc(P, &R->lin, (size_t)4 * N * N * N, s));
        PCHK(palloc(P, &R->grid, mo_grid_bytes(N, MO_LAYOUT_CELL), s));
        const size_t lb = mo_df_lazy_bytes(N);
        PCHK(palloc(P, &R->dfbits, lb, s));
        PCHK(cudaMemsetAsync(R->dfbits, 0, lb, s));
    } else {
    MoDfOptions opt;
    std::memset(&opt, 0, sizeof(opt));
    opt.method = R->method;
    opt.packet = R->packet;
    opt.band = R->band;
    const size_t sb = mo_df_build_scratch_bytes(q.ntv, q.ntf, N, R->method);
    void* scratch = nullptr;
    float* glin = nullptr;
    PCHK(palloc(P, &scratch, sb, s));
    PCHK(palloc(P, &glin, (size_t)4 * N * N * N, s));
    rc = mo_df_build_ex(tarV, q.ntv, tarF, q.ntf, N, R->params, &opt, scratch, sb, glin, R->status, sv);
    cudaFreeAsync(scratch, s);
    if (rc) {
        cudaFreeAsync(glin, s);
        return rc;
    }
    if (R->layout == MO_LAYOUT_LINEAR) {
        R->grid = glin;
    } else {
        PCHK(palloc(P, &R->grid, mo_grid_bytes(N, R->layout), s));
        rc = mo_grid_relayout(glin, N, R->layout, R->grid, sv);
        cudaFreeAsync(glin, s);
        if (rc) return rc;
    }
    }
    pfree(R->tarV, s);
    pfree(R->tarF, s);
    pfree(R->bbox, s);
    rc = mo_normalize(R->srcV, nv, R->params, 0, sv);
    if (rc) return rc;
    const size_t cb = mo_edge_csr_bytes(nv, nf, MO_EDGES_FACES);
    PCHK(palloc(P, &R->csr, cb, s));
    rc = mo_edge_csr_build(R->srcF, nf, MO_EDGES_FACES, nv, R->csr, cb, R->status + 1, sv);
    if (rc) return rc;
    pfree(R->srcF, s);
    R->nslices = (int)((nv + 31) / 32);
    PCHK(palloc(P, &R->slice_ptr, 4 * (size_t)(R->nslices + 1), s));
    rc = mo_sell_plan(R->csr, nv, 3 * nf, R->slice_ptr, sv);
    if (rc) return rc;
    PCHK(cudaMemcpyAsync(R->status + 2, R->slice_ptr + R->nslices, 4, cudaMemcpyDeviceToDevice, s));
    PCHK(cudaMemcpyAsync(R->host->status, R->status, 16, cudaMemcpyDeviceToHost, s));
    PCHK(cudaEventRecord(R->ev, s));
    R->phase = 1;
    R->state = MO_REQ_BUILDING;
    return MO_OK;
}

// Phase B: sliced-ELL records and the optimiser state (positions start at
// the normalised source, whose copy is also the rest pose of the offsets).
int phase_b(MoPool* P, Req* R) {
    const MoRequest& q = R->in;
    cudaStream_t s = R->stream;
    void* sv = reinterpret_cast<void*>(s);
    const int64_t nv = q.nv, nf = q.nf;
    const int64_t nrec = R->host->status[2];
    PCHK(palloc(P, &R->sell, 4 * (size_t)std::max<int64_t>(nrec, 1), s));
    int rc = mo_sell_fill(R->csr, nv, 3 * nf, R->slice_ptr, R->sell, sv);
    if (rc) return rc;
    pfree(R->csr, s);
    PCHK(palloc(P, &R->pos, 32 * (size_t)nv, s));
    PCHK(palloc(P, &R->rest, 16 * (size_t)nv, s));
    PCHK(palloc(P, &R->m, 12 * (size_t)nv, s));
    PCHK(palloc(P, &R->v, 12 * (size_t)nv, s));
    PCHK(cudaMemsetAsync(R->pos, 0, 32 * (size_t)nv, s));
    PCHK(cudaMemsetAsync(R->m, 0, 12 * (size_t)nv, s));
    PCHK(cudaMemsetAsync(R->v, 0, 12 * (size_t)nv, s));
    rc = mo_pack_pos(R->srcV, nv, R->pos, sv);
    if (!rc) rc = mo_pack_pos(R->srcV, nv, R->rest, sv);
    if (rc) return rc;
    pfree(R->srcV, s);
    R->ntiles = (R->nslices + R->spt - 1) / R->spt;
    if (R->lazy) {
        // the cells of the starting positions, before the first step
        fill_pair(P, R, &R->host->pair, 0);
        PCHK(palloc(P, &R->pair_dev, sizeof(MoPair), s));
        PCHK(cudaMemcpyAsync(R->pair_dev, &R->host->pair, sizeof(MoPair), cudaMemcpyHostToDevice, s));
        PCHK(palloc(P, &R->seedq, 72 * (size_t)nv + 16, s));
        int32_t* pq = R->seedq + 2 * nv;
        int32_t* cnt = pq + 16 * nv;
        PCHK(cudaMemsetAsync(cnt, 0, 8, s));
        rc = mo_df_lazy_seed(R->pair_dev, 0, R->pos, nv, R->seedq, pq, cnt, (int)nv, sv);
        if (!rc) rc = mo_df_lazy_fill(R->pair_dev, R->seedq, pq, cnt, (int)nv, P->fill_totals, sv);
        if (rc) return rc;
        pfree(R->seedq, s);
        pfree(R->pair_dev, s);
    }
    PCHK(cudaEventRecord(R->ev, s));
    R->phase = 2;
    return MO_OK;
}

void fill_pair(const MoPool* P, const Req* R, MoPair* p, int tile0) {
    std::memset(p, 0, sizeof(MoPair));
    p->grid = R->grid;
    p->slice_ptr = R->slice_ptr;
    p->sell = R->sell;
    p->rest = R->rest;
    p->pos0 = R->pos;
    p->pos1 = R->pos + 4 * R->in.nv;
    p->adam_m = R->m;
    p->adam_v = R->v;
    p->adam_tab = R->adam_tab;
    p->N = R->in.N;
    p->layout = R->layout;
    p->nv = (int32_t)R->in.nv;
    p->nslices = R->nslices;
    p->w_edge = R->in.w_edge;
    p->grad_scale = 1.0f;
    // torch.optim.Adam defaults, 1 - beta taken in double like its host code
    p->one_minus_b1 = (float)(1.0 - 0.9);
    p->b2 = (float)0.999;
    p->one_minus_b2 = (float)(1.0 - 0.999);
    p->eps = (float)1e-8;
    p->t0 = R->t;
    p->t_end = R->in.steps;
    p->tile0 = tile0;
    p->ntiles = R->ntiles;
    if (R->lazy) {
        const int N = R->in.N;
        const int64_t cell_words = ((int64_t)(N - 1) * (N - 1) * (N - 1) + 31) / 32;
        p->df_tree = R->tree;
        p->df_lin = R->lin;
        p->df_cells = R->dfbits;
        p->df_packets = R->dfbits + cell_words;
        p->df_status = R->status;
        p->df_queue = P->dfq;
        p->df_pqueue = P->dfpq;
        p->df_queue_count = P->dfq_count;
        p->df_ntri = (int32_t)R->in.ntf;
        p->df_queue_cap = P->dfq_cap;
        p->df_band = R->band;
    }
}

// Pair table (every group: t0 moves) and tile table (only when the active
// set changed) through a pinned double buffer on the step stream.
int upload(MoPool* P) {
    const int n = (int)P->active.size();
    const size_t pbytes = sizeof(MoPair) * (size_t)P->cfg.max_pairs;
    const int slot = P->slot;
    P->slot ^= 1;
    PCHK(cudaEventSynchronize(P->staging_ev[slot]));
    unsigned char* buf = P->staging[slot];
    MoPair* ptab = reinterpret_cast<MoPair*>(buf);
    MoTile* ttab = reinterpret_cast<MoTile*>(buf + pbytes);
    int32_t* nt = reinterpret_cast<int32_t*>(buf + pbytes + sizeof(MoTile) * (size_t)P->cfg.max_tiles);
    int tile0 = 0;
    for (int i = 0; i < n; ++i) {
        const Req* R = P->reqs[P->active[i]].get();
        fill_pair(P, R, &ptab[i], tile0);
        tile0 += R->ntiles;
    }
    PCHK(cudaMemcpyAsync(P->pairs_dev, ptab, sizeof(MoPair) * (size_t)n, cudaMemcpyHostToDevice, P->step));
    if (P->tiles_key != P->active) {
        int k = 0;
        for (int i = 0; i < n; ++i) {
            const Req* R = P->reqs[P->active[i]].get();
            for (int t = 0; t < R->ntiles; ++t, ++k) {
                ttab[k].pair = i;
                ttab[k].slice0 = t * R->spt;
                ttab[k].nslices = std::min(R->spt, R->nslices - t * R->spt);
                ttab[k].pad = 0;
            }
        }
        *nt = k;
        if (k) PCHK(cudaMemcpyAsync(P->tiles_dev, ttab, sizeof(MoTile) * (size_t)k, cudaMemcpyHostToDevice, P->step));
        PCHK(cudaMemcpyAsync(P->ntiles_dev, nt, 4, cudaMemcpyHostToDevice, P->step));
        P->tiles_key = P->active;
    }
    PCHK(cudaEventRecord(P->staging_ev[slot], P->step));
    return MO_OK;
}

int launch_steps(MoPool* P) {
    void* sv = reinterpret_cast<void*>(P->step);
    const bool lazy = P->cfg.df_mode == MO_DF_ON_DEMAND;
    if (lazy) PCHK(cudaMemsetAsync(P->dfq_count, 0, 8 * (size_t)P->cfg.group_steps, P->step));
    for (int k = 0; k < P->cfg.group_steps; ++k) {
        int rc = (lazy ? mo_fused_step_on_demand : mo_fused_step)(P->pairs_dev, P->tiles_dev, P->ntiles_dev,
                                                                  P->cfg.max_tiles, k, P->tile_loss,
                                                                  P->cfg.step_grid, sv);
        // the cells this step moved vertices into, before the next step reads them
        if (!rc && lazy)
            rc = mo_df_lazy_fill(P->pairs_dev, P->dfq, P->dfpq, P->dfq_count + 2 * k, P->dfq_cap, P->fill_totals, sv);
        if (rc) return rc;
    }
    return MO_OK;
}

// Capture the group of S launches once.  A warm-up launch with no tiles first
// loads the kernel outside the capture.
int capture(MoPool* P) {
    PCHK(cudaMemsetAsync(P->ntiles_dev, 0, 4, P->step));
    const bool lazy = P->cfg.df_mode == MO_DF_ON_DEMAND;
    int rc = (lazy ? mo_fused_step_on_demand : mo_fused_step)(P->pairs_dev, P->tiles_dev, P->ntiles_dev,
                                                              P->cfg.max_tiles, 0, P->tile_loss, 0,
                                                              reinterpret_cast<void*>(P->step));
    if (rc) return rc;
    PCHK(cudaStreamSynchronize(P->step));
    P->tiles_key.clear();  // the tile count was zeroed: re-send the table
    cudaGraph_t g = nullptr;
    PCHK(cudaStreamBeginCapture(P->step, cudaStreamCaptureModeThreadLocal));
    rc = launch_steps(P);
    cudaError_t e = cudaStreamEndCapture(P->step, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    PCHK(e);
    e = cudaGraphInstantiate(&P->graph, g, 0);
    cudaGraphDestroy(g);
    PCHK(e);
    return MO_OK;
}

int run_group(MoPool* P) {
    if (P->cfg.use_graph && !P->graph) {
        int rc = capture(P);
        if (rc) return rc;
    }
    int rc = upload(P);
    if (rc) return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (P->timing) {
        PCHK(cudaEventCreate(&e0));
        PCHK(cudaEventCreate(&e1));
        PCHK(cudaEventRecord(e0, P->step));
    }
    if (P->graph) {
        PCHK(cudaGraphLaunch(P->graph, P->step));
    } else {
        rc = launch_steps(P);
        if (rc) return rc;
    }
    P->stats.fused_launches += P->cfg.group_steps;
    const int n = (int)P->active.size();
    if (P->timing) {
        PCHK(cudaEventRecord(e1, P->step));
        double bytes = 0;
        for (int64_t id : P->active) {
            const Req* R = P->reqs[id].get();
            const int k = std::min(P->cfg.group_steps, R->in.steps - R->t);
            bytes += (double)k * (104.0 * (double)R->in.nv + 44.0 * 3.0 * (double)R->in.nf);
        }
        P->group_events.push_back({e0, e1});
        P->group_bytes.push_back(bytes);
    }
    // per-pair losses of this group's launches, when a pair retires (it keeps
    // the loss of its last step)
    bool retire = false;
    for (int64_t id : P->active) retire |= P->reqs[id]->t + P->cfg.group_steps >= P->reqs[id]->in.steps;
    if (retire) {
        rc = mo_pair_loss(P->pairs_dev, n, P->cfg.max_tiles, P->cfg.group_steps, P->tile_loss, P->pair_loss,
                          reinterpret_cast<void*>(P->step));
        if (rc) return rc;
    }
    P->stats.groups += 1;
    std::vector<int64_t> still;
    still.reserve(n);
    void* sv = reinterpret_cast<void*>(P->step);
    for (int i = 0; i < n; ++i) {
        const int64_t id = P->active[i];
        Req* R = P->reqs[id].get();
        const int k = std::min(P->cfg.group_steps, R->in.steps - R->t);
        R->t += k;
        if (R->t < R->in.steps) {
            still.push_back(id);
            continue;
        }
        const int64_t nv = R->in.nv;
        float* normed = R->result;
        float* denorm = R->result + 3 * nv;
        rc = mo_unpack_pos(R->pos + 4 * nv * (R->t & 1), nv, normed, sv);
        if (rc) return rc;
        PCHK(cudaMemcpyAsync(denorm, normed, 12 * nv, cudaMemcpyDeviceToDevice, P->step));
        rc = mo_normalize(denorm, nv, R->params, 1, sv);
        if (rc) return rc;
        // the loss (its buffer is rewritten by the next group) and the DF
        // status (on-demand fills report traversal faults there) on the step
        // stream; the result copies on the io stream, off the steps' path
        PCHK(cudaMemcpyAsync(&R->host->loss, P->pair_loss + (int64_t)(k - 1) * n + i, 8, cudaMemcpyDeviceToHost,
                             P->step));
        PCHK(cudaMemcpyAsync(R->host->status, R->status, 16, cudaMemcpyDeviceToHost, P->step));
        PCHK(cudaEventRecord(R->ev, P->step));
        PCHK(cudaStreamWaitEvent(P->io, R->ev, 0));
        const cudaMemcpyKind ok = R->in.out_on_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
        if (R->in.V_out) PCHK(cudaMemcpyAsync(R->in.V_out, denorm, 12 * nv, ok, P->io));
        if (R->in.V_normalized_out)
            PCHK(cudaMemcpyAsync(R->in.V_normalized_out, normed, 12 * nv, cudaMemcpyDeviceToDevice, P->io));
        PCHK(cudaEventRecord(R->ev, P->io));  // DONE when both streams' copies are
        free_state(R, P->step);
        R->phase = 4;
        P->retiring.push_back(id);
    }
    P->active.swap(still);
    return MO_OK;
}

int progress(MoPool* P) {
    // admission, FIFO, by bytes and slots; an idle pool always admits one
    while (!P->queued.empty() && (int)P->building.size() < P->cfg.max_building &&
           (int)(P->active.size() + P->building.size() + P->retiring.size()) < P->cfg.max_pairs) {
        Req* R = P->reqs[P->queued.front()].get();
        const size_t nb = estimate(R->in, R->layout, R->method, R->lazy);
        const bool idle = P->active.empty() && P->building.empty() && P->retiring.empty();
        if (P->stats.bytes_in_use + nb > P->cfg.hbm_budget_bytes && !idle) break;
        P->queued.pop_front();
        R->bytes = nb;
        P->stats.bytes_in_use += nb;
        P->stats.peak_bytes = std::max(P->stats.peak_bytes, P->stats.bytes_in_use);
        R->stream = P->builds[P->next_build++ % P->builds.size()];
        if (phase_a(P, R)) {
            fail(P, R, mo_last_error(), R->stream);
            continue;
        }
        P->building.push_back(R->id);
    }
    int tiles = 0;
    for (int64_t id : P->active) tiles += P->reqs[id]->ntiles;
    std::vector<int64_t> still;
    for (int64_t id : P->building) {
        Req* R = P->reqs[id].get();
        const cudaError_t q = cudaEventQuery(R->ev);
        if (q == cudaErrorNotReady) {
            still.push_back(id);
            continue;
        }
        PCHK(q);
        if (R->phase == 1) {
            if (R->host->status[0] || R->host->status[1]) {
                char msg[128];
                snprintf(msg, sizeof(msg), "invalid mesh (DF status %d, edge status %d)", R->host->status[0],
                         R->host->status[1]);
                fail(P, R, msg, R->stream);
                continue;
            }
            if (phase_b(P, R)) {
                fail(P, R, mo_last_error(), R->stream);
                continue;
            }
            still.push_back(id);
        } else if (R->ntiles > P->cfg.max_tiles) {
            fail(P, R, "request needs more tiles than the pool's max_tiles", R->stream);
        } else if (tiles + R->ntiles > P->cfg.max_tiles) {
            still.push_back(id);  // built; waits for tile room
        } else {
            PCHK(cudaStreamWaitEvent(P->step, R->ev, 0));
            R->phase = 3;
            R->state = MO_REQ_ACTIVE;
            tiles += R->ntiles;
            P->active.push_back(id);
        }
    }
    P->building.swap(still);
    if (!P->active.empty() && !P->hold) {
        int rc = run_group(P);
        if (rc) return rc;
    }
    still.clear();
    for (int64_t id : P->retiring) {
        Req* R = P->reqs[id].get();
        const cudaError_t q = cudaEventQuery(R->ev);
        if (q == cudaErrorNotReady) {
            still.push_back(id);
            continue;
        }
        PCHK(q);
        if (R->host->status[0]) {
            char msg[128];
            snprintf(msg, sizeof(msg), "distance-field fill failed (status %d)", R->host->status[0]);
            fail(P, R, msg, P->step);
            continue;
        }
        R->state = MO_REQ_DONE;
        P->stats.bytes_in_use -= R->bytes;
        R->bytes = 0;
        P->stats.done += 1;
        P->completed.push_back(id);
    }
    P->retiring.swap(still);
    P->stats.queued = (int32_t)P->queued.size();
    P->stats.building = (int32_t)P->building.size();
    P->stats.active = (int32_t)P->active.size();
    P->stats.retiring = (int32_t)P->retiring.size();
    int t2 = 0;
    for (int64_t id : P->active) t2 += P->reqs[id]->ntiles;
    P->stats.active_tiles = t2;
    P->stats.fill_launches_per_step = P->cfg.df_mode == MO_DF_ON_DEMAND ? 2 : 0;
    return MO_OK;
}

// Nothing to step: wait for the oldest build or retirement.
int block_idle(MoPool* P) {
    if (!P->active.empty() && !P->hold) return MO_OK;
    if (!P->building.empty()) PCHK(cudaEventSynchronize(P->reqs[P->building.front()]->ev));
    else if (!P->retiring.empty()) PCHK(cudaEventSynchronize(P->reqs[P->retiring.front()]->ev));
    return MO_OK;
}

int take_slot(MoPool* P, HostSlot** out) {
    if (P->free_slots.empty()) {
        const int n = 1024;
        HostSlot* chunk = nullptr;
        PCHK(cudaMallocHost(&chunk, sizeof(HostSlot) * n));
        P->slot_chunks.push_back(chunk);
        for (int i = n - 1; i >= 0; --i) P->free_slots.push_back(chunk + i);
    }
    *out = P->free_slots.back();
    P->free_slots.pop_back();
    std::memset(*out, 0, sizeof(HostSlot));
    return MO_OK;
}

// The request's host-side resources; its result goes back to the memory
// pool in stream order.
void destroy_req(MoPool* P, Req* R) {
    pfree(R->result, P->step);
    if (R->host) P->free_slots.push_back(R->host);
    R->host = nullptr;
    if (R->ev) cudaEventDestroy(R->ev);
    R->ev = nullptr;
}

}  // namespace
}  // namespace mo

using namespace mo;

namespace {
int init_pool(MoPool* P) {
    if (P->cfg.build_streams <= 0) P->cfg.build_streams = 2;
    if (P->cfg.max_building <= 0) P->cfg.max_building = 8;
    if (P->cfg.slices_per_tile <= 0 || P->cfg.slices_per_tile > MO_TILE_WARPS) P->cfg.slices_per_tile = MO_TILE_WARPS;
    PCHK(cudaGetDevice(&P->device));
    if (P->cfg.hbm_budget_bytes == 0) {
        size_t free_b = 0, total = 0;
        PCHK(cudaMemGetInfo(&free_b, &total));
        P->cfg.hbm_budget_bytes = (uint64_t)(0.6 * (double)free_b);
    }
    PCHK(cudaStreamCreateWithFlags(&P->step, cudaStreamNonBlocking));
    PCHK(cudaStreamCreateWithFlags(&P->io, cudaStreamNonBlocking));
    for (int i = 0; i < P->cfg.build_streams; ++i) {
        cudaStream_t s = nullptr;
        PCHK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        P->builds.push_back(s);
    }
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = P->device;
    PCHK(cudaMemPoolCreate(&P->mempool, &props));
    uint64_t keep = UINT64_MAX;  // keep freed blocks for later admissions
    PCHK(cudaMemPoolSetAttribute(P->mempool, cudaMemPoolAttrReleaseThreshold, &keep));
    const int S = P->cfg.group_steps;
    PCHK(cudaMalloc(&P->pairs_dev, sizeof(MoPair) * (size_t)P->cfg.max_pairs));
    PCHK(cudaMalloc(&P->tiles_dev, sizeof(MoTile) * (size_t)P->cfg.max_tiles));
    PCHK(cudaMalloc(&P->ntiles_dev, 4));
    PCHK(cudaMemset(P->ntiles_dev, 0, 4));
    PCHK(cudaMalloc(&P->tile_loss, sizeof(float) * (size_t)S * P->cfg.max_tiles * MO_TILE_WARPS));
    PCHK(cudaMalloc(&P->pair_loss, sizeof(double) * (size_t)S * P->cfg.max_pairs));
    if (P->cfg.df_mode == MO_DF_ON_DEMAND) {
        // a step queues at most one cell per vertex stepped
        const int64_t cap = (int64_t)P->cfg.max_tiles * 32 * MO_TILE_WARPS;
        MO_CHECK_ARG(cap < ((int64_t)1 << 28), "max_tiles too large for the on-demand cell queue");
        P->dfq_cap = (int)cap;
        PCHK(cudaMalloc(&P->dfq, 8 * (size_t)cap));
        PCHK(cudaMalloc(&P->dfpq, 64 * (size_t)cap));
        PCHK(cudaMalloc(&P->dfq_count, 8 * (size_t)S));
        PCHK(cudaMemset(P->dfq_count, 0, 8 * (size_t)S));
        PCHK(cudaMalloc(&P->fill_totals, 16));
        PCHK(cudaMemset(P->fill_totals, 0, 16));
    }
    const size_t sbytes = sizeof(MoPair) * (size_t)P->cfg.max_pairs + sizeof(MoTile) * (size_t)P->cfg.max_tiles + 16;
    for (int i = 0; i < 2; ++i) {
        PCHK(cudaMallocHost(&P->staging[i], sbytes));
        PCHK(cudaEventCreateWithFlags(&P->staging_ev[i], cudaEventDisableTiming));
        PCHK(cudaEventRecord(P->staging_ev[i], P->step));
    }
    PCHK(cudaDeviceSynchronize());
    return MO_OK;
}
}  // namespace

extern "C" int mo_pool_create(const MoPoolConfig* cfg, MoPool** out) {
    MO_CHECK_ARG(cfg && out, "null pointer");
    *out = nullptr;
    MO_CHECK_ARG(cfg->max_pairs > 0 && cfg->max_tiles > 0 && cfg->group_steps > 0, "bad pool sizes");
    MO_CHECK_ARG(mo_grid_bytes(64, cfg->layout) > 0, "unknown layout %d", cfg->layout);
    MO_CHECK_ARG(cfg->df_mode == MO_DF_FULL || cfg->df_mode == MO_DF_ON_DEMAND, "unknown df_mode %d", cfg->df_mode);
    MoPool* P = new MoPool();
    P->cfg = *cfg;
    const int rc = init_pool(P);
    if (rc) {
        mo_pool_destroy(P);
        return rc;
    }
    *out = P;
    return MO_OK;
}

extern "C" int mo_pool_submit(MoPool* P, const MoRequest* q, int64_t* id_out) {
    MO_CHECK_ARG(P && q && id_out, "null pointer");
    MO_CHECK_ARG(q->nv > 0 && q->nf >= 0 && q->ntv > 0 && q->ntf > 0, "empty mesh");
    MO_CHECK_ARG(q->srcV && q->tarV && q->tarF && (q->nf == 0 || q->srcF), "null mesh pointer");
    MO_CHECK_ARG(q->N >= 2 && q->N <= 1024 && q->steps > 0, "bad grid resolution %d or step count %d", q->N,
                 q->steps);
    MO_CHECK_ARG(q->nv < ((int64_t)1 << 31) && 3 * q->nf < ((int64_t)1 << 30), "mesh too large");
    MO_CHECK_ARG(q->lr > 0 && std::isfinite(q->lr), "bad learning rate");
    std::unique_ptr<Req> R(new Req());
    R->in = *q;
    R->layout = q->layout >= 0 ? q->layout : P->cfg.layout;
    MO_CHECK_ARG(mo_grid_bytes(q->N, R->layout) > 0, "unknown layout %d", R->layout);
    R->lazy = P->cfg.df_mode == MO_DF_ON_DEMAND;
    if (R->lazy) R->layout = MO_LAYOUT_CELL;  // the fills write cell records
    R->spt = (q->slices_per_tile > 0 && q->slices_per_tile <= MO_TILE_WARPS) ? q->slices_per_tile
                                                                            : P->cfg.slices_per_tile;
    MO_CHECK_ARG(q->df_method == MO_DF_AUTO || q->df_method == MO_DF_BRUTE || q->df_method == MO_DF_LBVH,
                 "unknown DF method %d", q->df_method);
    MO_CHECK_ARG(q->df_packet >= MO_PACKET_4x4x2 && q->df_packet <= MO_PACKET_LAST, "unknown packet %d",
                 q->df_packet);
    R->method = q->df_method == MO_DF_AUTO ? mo_df_method_for(q->ntf, q->N) : q->df_method;
    R->packet = q->df_packet;
    MO_CHECK_ARG(q->df_band <= 4.0f && q->df_band == q->df_band, "bad DF band %g", (double)q->df_band);
    R->band = q->df_band < 0.0f ? mo_df_loss_band(q->N) : q->df_band;
    int rc = adam_table(P, q->lr, q->steps, &R->adam_tab);
    if (rc) return rc;
    R->id = P->next_id++;
    PCHK(cudaEventCreateWithFlags(&R->ev, cudaEventDisableTiming));
    rc = take_slot(P, &R->host);
    if (rc) return rc;
    PCHK(palloc(P, &R->result, 24 * (size_t)q->nv, P->step));
    *id_out = R->id;
    P->queued.push_back(R->id);
    P->reqs[R->id] = std::move(R);
    P->stats.submitted += 1;
    P->stats.queued = (int32_t)P->queued.size();
    return MO_OK;
}

extern "C" int mo_pool_progress(MoPool* P, int block, int64_t* n_finished_out) {
    MO_CHECK_ARG(P, "null pool");
    int rc = progress(P);
    if (!rc && block) rc = block_idle(P);
    if (n_finished_out) *n_finished_out = P->stats.done + P->stats.failed;
    return rc;
}

extern "C" int mo_pool_wait(MoPool* P) {
    MO_CHECK_ARG(P, "null pool");
    while (P->stats.done + P->stats.failed < P->stats.submitted) {
        if (P->hold && P->building.empty()) {
            if (P->queued.empty()) break;  // all built, held
            const size_t before = P->queued.size();
            int rc = progress(P);
            if (rc) return rc;
            MO_CHECK_ARG(P->queued.size() < before || !P->building.empty(),
                         "pool on hold: %zu requests cannot be admitted (max_pairs or the HBM budget)",
                         P->queued.size());
            continue;
        }
        int rc = progress(P);
        if (!rc) rc = block_idle(P);
        if (rc) return rc;
    }
    PCHK(cudaStreamSynchronize(P->step));
    return MO_OK;
}

extern "C" int mo_pool_completed(MoPool* P, int64_t* ids, int max_ids, int* n_out) {
    MO_CHECK_ARG(P && n_out && (ids || max_ids == 0) && max_ids >= 0, "bad arguments");
    int n = 0;
    while (n < max_ids && !P->completed.empty()) {
        ids[n++] = P->completed.front();
        P->completed.pop_front();
    }
    *n_out = n;
    return MO_OK;
}

extern "C" int mo_pool_state(MoPool* P, int64_t id, int32_t* state_out) {
    MO_CHECK_ARG(P && state_out, "null pointer");
    auto it = P->reqs.find(id);
    MO_CHECK_ARG(it != P->reqs.end(), "unknown request %lld", (long long)id);
    *state_out = it->second->state;
    return MO_OK;
}

extern "C" int mo_pool_error(MoPool* P, int64_t id, char* buf, size_t buf_bytes) {
    MO_CHECK_ARG(P && buf && buf_bytes > 0, "bad arguments");
    auto it = P->reqs.find(id);
    MO_CHECK_ARG(it != P->reqs.end(), "unknown request %lld", (long long)id);
    snprintf(buf, buf_bytes, "%s", it->second->error);
    return MO_OK;
}

extern "C" int mo_pool_result(MoPool* P, int64_t id, float* V_out, float* V_normalized_out, int out_on_host,
                              double* loss_out) {
    MO_CHECK_ARG(P, "null pool");
    auto it = P->reqs.find(id);
    MO_CHECK_ARG(it != P->reqs.end(), "unknown request %lld", (long long)id);
    Req* R = it->second.get();
    if (R->state == MO_REQ_FAILED) {
        set_error("request %lld failed: %s", (long long)id, R->error);
        return MO_ERR_DEVICE;
    }
    MO_CHECK_ARG(R->state == MO_REQ_DONE, "request %lld is not finished", (long long)id);
    const size_t bytes = 12 * (size_t)R->in.nv;
    const cudaMemcpyKind kind = out_on_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    // the retirement is complete (DONE); copy on the pool's I/O stream and wait
    // for just these copies, so the result memory can be recycled afterwards
    if (V_out) PCHK(cudaMemcpyAsync(V_out, R->result + 3 * R->in.nv, bytes, kind, P->io));
    if (V_normalized_out) PCHK(cudaMemcpyAsync(V_normalized_out, R->result, bytes, kind, P->io));
    if (V_out || V_normalized_out) PCHK(cudaStreamSynchronize(P->io));
    if (loss_out) *loss_out = R->host->loss;
    return MO_OK;
}

extern "C" int mo_pool_release(MoPool* P, int64_t id) {
    MO_CHECK_ARG(P, "null pool");
    auto it = P->reqs.find(id);
    MO_CHECK_ARG(it != P->reqs.end(), "unknown request %lld", (long long)id);
    Req* R = it->second.get();
    MO_CHECK_ARG(R->state == MO_REQ_DONE || R->state == MO_REQ_FAILED, "request %lld is still running",
                 (long long)id);
    PCHK(cudaEventSynchronize(R->ev));
    destroy_req(P, R);
    P->reqs.erase(it);
    return MO_OK;
}

extern "C" int mo_pool_set_hold(MoPool* P, int hold) {
    MO_CHECK_ARG(P, "null pool");
    P->hold = hold != 0;
    return MO_OK;
}

extern "C" int mo_pool_set_timing(MoPool* P, int enable) {
    MO_CHECK_ARG(P, "null pool");
    P->timing = enable != 0;
    return MO_OK;
}

extern "C" int mo_pool_run_groups(MoPool* P, int groups) {
    MO_CHECK_ARG(P && groups >= 0, "bad arguments");
    for (int g = 0; g < groups && !P->active.empty(); ++g) {
        int rc = run_group(P);
        if (rc) return rc;
    }
    return MO_OK;
}

extern "C" int mo_pool_group_time(MoPool* P, double* ms_out, double* bytes_out) {
    MO_CHECK_ARG(P && ms_out && bytes_out, "null pointer");
    PCHK(cudaStreamSynchronize(P->step));
    double ms = 0, bytes = 0;
    for (size_t i = 0; i < P->group_events.size(); ++i) {
        float t = 0;
        PCHK(cudaEventElapsedTime(&t, P->group_events[i].first, P->group_events[i].second));
        ms += t;
        bytes += P->group_bytes[i];
    }
    for (auto& ge : P->group_events) {
        cudaEventDestroy(ge.first);
        cudaEventDestroy(ge.second);
    }
    P->group_events.clear();
    P->group_bytes.clear();
    *ms_out = ms;
    *bytes_out = bytes;
    return MO_OK;
}

extern "C" int mo_pool_stats(MoPool* P, MoPoolStats* out) {
    MO_CHECK_ARG(P && out, "null pointer");
    *out = P->stats;
    return MO_OK;
}

extern "C" int mo_pool_fill_totals(MoPool* P, int64_t* out2) {
    MO_CHECK_ARG(P && out2, "null pointer");
    out2[0] = out2[1] = 0;
    if (!P->fill_totals) return MO_OK;
    PCHK(cudaStreamSynchronize(P->step));
    for (cudaStream_t s : P->builds) PCHK(cudaStreamSynchronize(s));
    PCHK(cudaMemcpy(out2, P->fill_totals, 16, cudaMemcpyDeviceToHost));
    return MO_OK;
}

extern "C" int mo_pool_trim(MoPool* P, uint64_t keep_bytes) {
    MO_CHECK_ARG(P, "null pool");
    PCHK(cudaStreamSynchronize(P->step));
    for (cudaStream_t s : P->builds) PCHK(cudaStreamSynchronize(s));
    PCHK(cudaMemPoolTrimTo(P->mempool, (size_t)keep_bytes));
    return MO_OK;
}

extern "C" int mo_pool_step_stream(MoPool* P, void** stream_out) {
    MO_CHECK_ARG(P && stream_out, "null pointer");
    *stream_out = reinterpret_cast<void*>(P->step);
    return MO_OK;
}

extern "C" int mo_pool_destroy(MoPool* P) {
    if (!P) return MO_OK;
    cudaStreamSynchronize(P->step);
    for (cudaStream_t s : P->builds) cudaStreamSynchronize(s);
    for (auto& kv : P->reqs) free_state(kv.second.get(), P->step);
    cudaStreamSynchronize(P->step);
    for (auto& kv : P->reqs) destroy_req(P, kv.second.get());
    P->reqs.clear();
    cudaStreamSynchronize(P->step);
    for (mo::HostSlot* c : P->slot_chunks) cudaFreeHost(c);
    for (auto& a : P->adam_tabs) cudaFree(a.dev);
    if (P->graph) cudaGraphExecDestroy(P->graph);
    cudaFree(P->pairs_dev);
    cudaFree(P->dfq);
    cudaFree(P->dfpq);
    cudaFree(P->fill_totals);
    cudaFree(P->dfq_count);
    cudaFree(P->tiles_dev);
    cudaFree(P->ntiles_dev);
    cudaFree(P->tile_loss);
    cudaFree(P->pair_loss);
    for (int i = 0; i < 2; ++i) {
        if (P->staging[i]) cudaFreeHost(P->staging[i]);
        if (P->staging_ev[i]) cudaEventDestroy(P->staging_ev[i]);
    }
    for (auto& ge : P->group_events) {
        cudaEventDestroy(ge.first);
        cudaEventDestroy(ge.second);
    }
    if (P->mempool) cudaMemPoolDestroy(P->mempool);
    for (cudaStream_t s : P->builds) cudaStreamDestroy(s);
    if (P->io) cudaStreamDestroy(P->io);
    if (P->step) cudaStreamDestroy(P->step);
    delete P;
    return MO_OK;
}
