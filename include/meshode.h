/*
 * meshode.h -- C ABI of libmeshode.so, the GB300 (sm_103a) implementation of
 * MeshODE's per-iteration deformation hot path.
 *
 * Conventions
 *   - Every entry point returns an int status (MO_OK == 0); on failure
 *     mo_last_error() returns a message for the calling thread.
 *   - Every pointer argument is a DEVICE pointer owned by the caller unless
 *     the comment says "host".  `stream` is a cudaStream_t (NULL = legacy
 *     default stream).  All calls are asynchronous on `stream` unless stated.
 *   - Vertex arrays are float32 [n,3] row-major (the layout of the reference's
 *     torch tensors); faces int32 [m,3]; edge lists int32 [k,2].
 *   - Distance grids in MO_LAYOUT_LINEAR are float32 [N][N][N] indexed
 *     [z][y][x] like UniformGrid::voxel_distance_ (src/lib/uniformgrid.h:33).
 *   - The step path (loss, gradient, Adam, fused step) allocates nothing;
 *     builders take caller scratch (or NULL: then the library allocates it
 *     stream-ordered and frees it before returning).
 */
#ifndef MESHODE_GB300_H_
#define MESHODE_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MO_OK 0
#define MO_ERR_INVALID 1 /* bad argument (checked on the host) */
#define MO_ERR_CUDA 2    /* CUDA runtime error */
#define MO_ERR_SCRATCH 3 /* caller scratch too small */
#define MO_ERR_DEVICE 4  /* a kernel reported an error through its status word */

#define MO_LAYOUT_LINEAR 0 /* [z][y][x] float, 4*N^3 bytes */
#define MO_LAYOUT_CELL 1   /* per cell (x,y,z < N-1) its 8 corners, 32 B = one sector */
#define MO_LAYOUT_BRICK4 2 /* 4x4x4 bricks of 256 B, bricks and voxels [z][y][x], N padded to 4 */

#define MO_DF_AUTO 0
#define MO_DF_BRUTE 1 /* shared-memory-tiled brute force (small targets) */
#define MO_DF_LBVH 2  /* Morton codes + radix sort + Karras LBVH + warp packet traversal */

#define MO_EDGES_FACES 0 /* idx = F[m,3]; half-edge 3f+j = (F[f][j], F[f][(j+1)%3]) */
#define MO_EDGES_LIST 1  /* idx = E[k,2]; edge k = (E[k][0], E[k][1]) */

/* Message describing the last failure on this host thread. */
const char* mo_last_error(void);
/* Library ABI version (major*100 + minor). */
int mo_version(void);
/* Kernel launches issued by this library since it was loaded (launches
 * replayed from a captured CUDA graph are not included). */
unsigned long long mo_launch_count(void);

/* ------------------------------------------------------------------------
 * Normalisation by the target's transform.
 * Replaces Mesh::Normalize (src/lib/mesh.cc:66-96), NormalizeByTemplate and
 * DenormalizeByTemplate (src/interface/normalize.cc:5-45).
 * ------------------------------------------------------------------------ */
/* Exact per-axis min/max of V into bbox6 (device int32[6], ordered-int
 * encoding: min x,y,z then max x,y,z).  NaNs are ignored. */
int mo_bbox(const float* V, int64_t n, int32_t* bbox6, void* stream);
/* params4 (device double[4]) = {scale, tx, ty, tz}:
 * scale = 1.1 * longest extent, t = min - 0.05*scale (mesh.cc:79-82). */
int mo_norm_params(const int32_t* bbox6, double* params4, void* stream);
/* In place: v = (v - t)/scale (inverse == 0) or v = v*scale + t
 * (inverse != 0), evaluated in double and rounded to float like
 * normalize.cc:21 and :42. */
int mo_normalize(float* V, int64_t n, const double* params4, int inverse, void* stream);

/* ------------------------------------------------------------------------
 * Distance-field build.  Replaces Mesh::ConstructDistanceField
 * (src/lib/mesh.cc:106-152) and its igl::point_mesh_squared_distance query
 * (mesh.cc:140): grid[z][y][x] = unsigned distance from (x/N, y/N, z/N) to the
 * nearest triangle of the target normalised by params4.
 * ------------------------------------------------------------------------ */
size_t mo_df_build_scratch_bytes(int64_t nv, int64_t nf, int N, int method);
/* status_out: optional device int32.  When given, the call does not
 * synchronise; bit 0 (a face index outside [0, nv)) and bit 1 (traversal
 * stack overflow) are OR-ed into it for the caller to read later.  When NULL
 * the call synchronises `stream` and reports those as MO_ERR_DEVICE. */
int mo_df_build(const float* V, int64_t nv, const int32_t* F, int64_t nf, int N,
                const double* params4, int method, void* scratch, size_t scratch_bytes,
                float* grid_linear_out, int32_t* status_out, void* stream);
/* The LBVH stages of mo_df_build on their own, for checking against a CPU
 * build of the same codes: sorted 30-bit Morton codes of the triangle
 * centroids (uint32[nf]), the stable sort permutation (int32[nf]), the Karras
 * children of the nf-1 internal nodes (>= 0 internal, ~leaf for leaves) and
 * the root box (float[6], lo then hi; for nf > 1).  Synchronises `stream`. */
int mo_lbvh_build(const float* V, int64_t nv, const int32_t* F, int64_t nf, const double* params4,
                  void* scratch, size_t scratch_bytes, uint32_t* sorted_codes, int32_t* order,
                  int32_t* left, int32_t* right, float* root_box, void* stream);
/* Allocation-free variant of mo_df_build, for callers that cannot allocate
 * device memory while they run (a plugin inside a host runtime that owns the
 * device memory pool, a real-time loop that forbids allocation after
 * start-up).  No counterpart in the reference.  The build's scratch is one
 * fixed device array of MO_DF_NOALLOC_SCRATCH_BYTES that every GPU loading
 * this library holds until the process exits; targets whose scratch need
 * (mo_df_build_scratch_bytes with mo_df_method_for's method) exceeds it are
 * rejected with MO_ERR_SCRATCH.  The LBVH build needs about 405 bytes per
 * triangle plus 12 per vertex, so the array holds targets of up to 20,000
 * triangles with up to 10,000 vertices (a closed mesh has about half as
 * many vertices as triangles).  The caller still passes the inputs and the
 * output grid.  The first call on a device, made with that device current,
 * looks up the array's device address (under lazy module loading that may
 * also be when the array is placed in device memory) and caches it: make one
 * warm-up call per device at start-up, before the phase that must not
 * allocate, and do not use the library across a cudaDeviceReset.  The call
 * cannot be made during stream capture: it copies the build status to the
 * host and synchronises `stream`.  Every call shares the array and leaves
 * its contents behind: calls that overlap on the GPU (other streams, other
 * host threads) race and must be serialised by the caller. */
#define MO_DF_NOALLOC_SCRATCH_BYTES (8u << 20)
int mo_df_build_noalloc(const float* V, int64_t nv, const int32_t* F, int64_t nf, int N,
                        const double* params4, float* grid_linear_out, void* stream);
/* MO_DF_NOALLOC_SCRATCH_BYTES as compiled into the library. */
size_t mo_df_noalloc_scratch_capacity(void);
/* Traversal packet shapes: the 32 voxels one warp walks the tree with. */
#define MO_PACKET_4x4x2 0
#define MO_PACKET_8x4x1 1
#define MO_PACKET_4x2x4 2
#define MO_PACKET_2x4x4 3
#define MO_PACKET_8x2x2 4
/* Two voxels per lane (64 per warp, the second one PZ further along z),
 * evaluated with packed FP32 math: bases 4x4x2, 2x4x4 and 8x4x1. */
#define MO_PACKET_4x4x4 5
#define MO_PACKET_2x4x8 6
#define MO_PACKET_8x4x2 7
/* One voxel per lane, a bucket's triangles tested two at a time with packed
 * FP32 math (for dense targets). */
#define MO_PACKET_4x4x2_TRI2 8
#define MO_PACKET_2x4x4_TRI2 9
#define MO_PACKET_LAST 9
typedef struct MoDfOptions {
    int32_t method;   /* MO_DF_AUTO, MO_DF_BRUTE or MO_DF_LBVH */
    int32_t packet;   /* MO_PACKET_* for MO_DF_LBVH */
    float band;       /* 0: exact grid.  > 0: voxels at distance >= band store
                       * band, except in the two lowest layers along each axis
                       * (x, y or z <= 1), whose band is band + 13/N; see
                       * mo_df_loss_band */
    int32_t reserved; /* 0 */
} MoDfOptions;
/* mo_df_build with explicit build options (opt == NULL: defaults).  method
 * and packet change only the speed, never the grid. */
int mo_df_build_ex(const float* V, int64_t nv, const int32_t* F, int64_t nf, int N,
                   const double* params4, const MoDfOptions* opt, void* scratch, size_t scratch_bytes,
                   float* grid_linear_out, int32_t* status_out, void* stream);
/* mo_df_build_ex that also measures the work of the nearest-triangle search:
 * counts (device uint64[2], accumulated into, not cleared) += the node
 * visits and the point-triangle tests of the build, each counted per voxel
 * (a warp's visit counts once for every voxel it walks for).  The brute
 * force counts N^3 * nf tests and no visits.  The grid is the same as
 * mo_df_build_ex's; the counting build runs slower and is for measurement
 * only.  No counterpart in the reference. */
int mo_df_build_count(const float* V, int64_t nv, const int32_t* F, int64_t nf, int N,
                      const double* params4, const MoDfOptions* opt, void* scratch, size_t scratch_bytes,
                      float* grid_linear_out, int32_t* status_out, uint64_t* counts, void* stream);
/* The smallest band that leaves DistanceFieldLoss unchanged for every input:
 * 0.2 + sqrt(3)/N + 1e-3.  UniformGrid::DistanceFloat (uniformgrid.cc:
 * 147-148) returns 0 when the in-range trilinear value exceeds 0.2; grid
 * values are 1-Lipschitz, so a cell with a corner at or beyond the band has
 * every corner above 0.2 + 1e-3 - rounding and interpolates above 0.2 from
 * either grid.  The only lookups that extrapolate (coordinates in (-1/N, 0))
 * read cells whose 8 corners all lie in the two lowest layers of an axis;
 * there, with corners 1/N apart differing by at most 1/N, each extrapolated
 * axis (weights in (-1, 0)) lowers the value by at most the spread of its
 * inputs and triples their spread, so the value is at least the smallest
 * corner minus (1 + 3 + 9)/N, and those layers use band + 13/N.  The
 * serving pool builds with this band: its losses and results are
 * bit-identical to an exact grid's, and the build skips most of the far
 * field. */
float mo_df_loss_band(int N);
/* The target's traversal tree alone, for on-demand fills (mo_df_lazy_fill):
 * the steps of the LBVH build of mo_df_build_ex without the grid pass.
 * tree_out (mo_df_tree_bytes(nf) bytes, 16-byte aligned; 128-byte aligned
 * puts every node record in one cache line) gets the sorted triangle
 * records (80 B each), padded to a multiple of 128 B, then the internal
 * nodes' traversal records (128 B each); nf <= 2^27.  scratch:
 * mo_df_tree_scratch_bytes; status_out (device int32) gets bit 1 for a face
 * index out of range.  Nothing is synchronised. */
size_t mo_df_tree_bytes(int64_t nf);
size_t mo_df_tree_scratch_bytes(int64_t nv, int64_t nf);
int mo_df_tree_build(const float* V, int64_t nv, const int32_t* F, int64_t nf, const double* params4,
                     void* scratch, size_t scratch_bytes, void* tree_out, int32_t* status_out, void* stream);
/* Method MO_DF_AUTO resolves to (host-side heuristic, exported for tests). */
int mo_df_method_for(int64_t nf, int N);

/* Bytes of a grid in `layout`; 0 for an invalid layout. */
size_t mo_grid_bytes(int N, int layout);
/* Re-lay a linear grid into `layout` (MO_LAYOUT_CELL packs each cell's 8
 * corners contiguously so one trilinear lookup reads one 32-byte sector). */
int mo_grid_relayout(const float* grid_linear, int N, int layout, float* out, void* stream);

/* ------------------------------------------------------------------------
 * DistanceFieldLoss.  Replaces DistanceFieldLoss_forward
 * (src/interface/distance_layer.cc:8-37, per vertex d(v)^2 with
 * UniformGrid::DistanceFloat, src/lib/uniformgrid.cc:85-150) and
 * DistanceFieldLoss_backward (distance_layer.cc:39-81, d * grad d through
 * ceres::Jet<float,3>).  Bit-identical to the reference's float arithmetic.
 * ------------------------------------------------------------------------ */
int mo_dfloss_forward(const float* V, int64_t n, const float* grid, int N, int layout,
                      float* loss_out, void* stream);
int mo_dfloss_backward(const float* V, int64_t n, const float* grid, int N, int layout,
                       float* grad_out, void* stream);
/* Both in one pass.  loss_out may be NULL.  If use_mask != 0 the gradient of
 * vertex i is multiplied by (0.5*loss_i < mask_thresh), the d < 0.03 mask of
 * GraphLossFunction (src/python/layers/graph_loss_layer.py:18,40). */
int mo_dfloss_fwd_bwd(const float* V, int64_t n, const float* grid, int N, int layout,
                      float* loss_out, float* grad_out, int use_mask, float mask_thresh,
                      void* stream);

/* ------------------------------------------------------------------------
 * Edge (rigidity) losses.  Replaces StoreRigidityInformation /
 * RigidEdgeLoss_forward / RigidEdgeLoss_backward (src/interface/rigid_layer.cc:
 * 11-46, 48-89, 91-133) and StoreGraphInformation / GraphEdgeLoss_*
 * (src/interface/graph_layer.cc:11-135).  The backward scatter is a
 * deterministic per-vertex reduction over a vertex -> half-edge CSR whose
 * entries are in half-edge order, which reproduces the reference's serial
 * scatter bit for bit.
 * ------------------------------------------------------------------------ */
int64_t mo_edge_count(int64_t n_items, int kind);
/* off_out [H,3] = v1 - v0 (rigid_layer.cc:29-45, graph_layer.cc:18-32). */
int mo_edge_offsets(const float* V, int64_t nv, const int32_t* idx, int64_t n_items, int kind,
                    float* off_out, void* stream);
/* loss_out [H,3] = (v1 - v0 - off)^2 per component (rigid_layer.cc:72-86). */
int mo_edge_forward(const float* V, int64_t nv, const int32_t* idx, int64_t n_items, int kind,
                    const float* off, float* loss_out, void* stream);
/* Bytes of the CSR buffer for nv vertices and the given half-edge list. */
size_t mo_edge_csr_bytes(int64_t nv, int64_t n_items, int kind);
/* Validates 0 <= index < nv on the device.  status_out: optional device
 * int32; when given, the call does not synchronise and bit 0 is OR-ed into it
 * for an out-of-range index.  When NULL the call synchronises `stream` and
 * returns MO_ERR_DEVICE for an out-of-range index. */
int mo_edge_csr_build(const int32_t* idx, int64_t n_items, int kind, int64_t nv, void* csr,
                      size_t csr_bytes, int32_t* status_out, void* stream);
/* grad_out [nv,3] = sum over incident half-edges of -/+ (v1 - v0 - off)
 * (rigid_layer.cc:113-130). */
int mo_edge_backward(const float* V, int64_t nv, const void* csr, int64_t nh, const float* off,
                     float* grad_out, void* stream);

/* Weighted edges.  Replaces StoreCadInformation / CadEdgeLoss_forward /
 * CadEdgeLoss_backward (src/interface/cad_layer.cc:11-223).  The CAD loss's
 * edge set is E's edges followed by F's half-edges: list_out [ne+3nf, 2]
 * (cad_layer.cc:33-67).  Its rest offsets come from mo_edge_offsets over that
 * list (MO_EDGES_LIST), its weights lambda_out [H] =
 * 2e-2 / (|off| + 1e-8) (cad_layer.cc:48-49, 71-72: the float norm, then
 * double, rounded to float). */
int mo_edge_cad_list(const int32_t* E, int64_t ne, const int32_t* F, int64_t nf, int32_t* list_out,
                     void* stream);
int mo_edge_cad_weights(const float* off, int64_t nh, float* lambda_out, void* stream);
/* mo_edge_forward / mo_edge_backward with a per-edge weight w [H] (NULL: the
 * unweighted calls): loss_out [H,3] = ((v1 - v0 - off) * w)^2 per component
 * (cad_layer.cc:114-122); grad_out [nv,3] = the serial scatter of
 * (v1 - v0 - off) * (w * w) (cad_layer.cc:195-202). */
int mo_edge_forward_w(const float* V, int64_t nv, const int32_t* idx, int64_t n_items, int kind,
                      const float* off, const float* w, float* loss_out, void* stream);
int mo_edge_backward_w(const float* V, int64_t nv, const void* csr, int64_t nh, const float* off,
                       const float* w, float* grad_out, void* stream);
/* One evaluation of the edge term: loss_out [H,3] as mo_edge_forward_w
 * (NULL: not computed) and grad_out [nv,3] as mo_edge_backward_w, for the
 * half-edges of idx (kind) whose CSR (mo_edge_csr_build over the same idx)
 * is csr; w NULL: weight 1 (RigidEdgeLoss / GraphEdgeLoss), else the
 * CadEdgeLoss weights.  Same results as the two calls. */
int mo_edge_fwd_bwd(const float* V, int64_t nv, const int32_t* idx, int64_t n_items, int kind, const void* csr,
                    const float* off, const float* w, float* loss_out, float* grad_out, void* stream);

/* Sliced-ELL (32-vertex slices, column-major records) view of the CSR for
 * the fused step: one int32 record per incident half-edge, other | role<<31
 * (role 1 when the vertex is the half-edge's v1), in half-edge order;
 * padding records are -1.  The fused step recomputes each rest offset as
 * rest[v1] - rest[v0] from the rest positions, the same single subtraction
 * StoreRigidityInformation makes.  slice_ptr is int32[ceil(nv/32)+1];
 * mo_sell_plan fills it asynchronously, the record count ending up in
 * slice_ptr[ceil(nv/32)] (read it before sizing the records for
 * mo_sell_fill). */
int mo_sell_plan(const void* csr, int64_t nv, int64_t nh, int32_t* slice_ptr, void* stream);
int mo_sell_fill(const void* csr, int64_t nv, int64_t nh, const int32_t* slice_ptr, int32_t* records,
                 void* stream);
/* Per-edge weights w [H] laid out like the records (record_w: as many floats
 * as records; padding 0), for the weighted fused step (MoPair.sell_w). */
int mo_sell_fill_w(const void* csr, int64_t nv, int64_t nh, const int32_t* slice_ptr, const float* w,
                   float* record_w, void* stream);

/* ------------------------------------------------------------------------
 * Adam.  Replaces torch.optim.Adam([V], lr) in the reference's loops
 * (src/python/rigid_deform.py:32,39): the update of
 * torch/optim/adam.py _single_tensor_adam (lerp, mul/addcmul,
 * sqrt/bias-correction, addcdiv) with step_size = lr/(1-b1^t) and
 * bc2_sqrt = sqrt(1-b2^t) computed by the caller in double.
 * ------------------------------------------------------------------------ */
int mo_adam_step(float* P, const float* G, float* M, float* Vsq, int64_t n, float one_minus_b1,
                 float b2, float one_minus_b2, float eps, float step_size, float bc2_sqrt,
                 void* stream);

/* ------------------------------------------------------------------------
 * Fused optimiser step over many deformation pairs (serving).  One launch =
 * one Adam step of every active pair: DF loss+gradient, edge residuals and
 * their CSR-ordered gradient, optional mask/weights, Adam, and the per-tile
 * loss partial.  Replaces the per-iteration body of rigid_deform.py:35-39 /
 * cad_deform.py:30-35 (RigidLossFunction / GraphLossFunction + Adam).
 * All descriptors live in device memory so a captured CUDA graph of these
 * launches stays valid while pairs are admitted and retired.
 * ------------------------------------------------------------------------ */
typedef struct MoPair {
    const float* grid;      /* layout-specific grid */
    const int32_t* slice_ptr;
    const int32_t* sell;    /* sliced-ELL records (mo_sell_fill) */
    const float* rest;      /* float4 [nv] rest positions the offsets are taken from */
    float* pos0;            /* float4 [nv] positions, even steps read pos0 */
    float* pos1;            /* float4 [nv] positions, odd steps read pos1 */
    float* adam_m;          /* float [nv*3] */
    float* adam_v;          /* float [nv*3] */
    const float* adam_tab;  /* float2 [tmax]: (step_size, bc2_sqrt) of step t at index t-1 */
    float* grad_dbg;        /* optional float [nv*3]: total gradient of each step */
    int32_t N, layout, nv, nslices;
    float w_edge;           /* edge-loss weight (1, lambda^2 or rigidity^2) */
    float mask_thresh;      /* DF gradient mask threshold on 0.5*d^2 */
    int32_t use_mask;
    float grad_scale;       /* upstream gradient grad_h */
    float one_minus_b1, b2, one_minus_b2, eps;
    int32_t t0;             /* steps completed before this group of launches */
    int32_t t_end;          /* last step to run */
    int32_t tile0, ntiles;  /* the pair's contiguous range in the MoTile array */
    /* On-demand distance field (df_cells != NULL, MO_LAYOUT_CELL only): a
     * cell of `grid` is written by mo_df_lazy_fill before any step reads it.
     * A step that moves a vertex into a cell whose bit is not yet set sets
     * it and queues the cell (df_queue), and queues every voxel packet the
     * cell's corners lie in whose bit is not yet set (df_pqueue); counters
     * df_queue_count[2k] (cells) and [2k+1] (packets) for launch index k.
     * The fill launched after that step computes the packets, then writes
     * the cells, so the next step finds them.  Every voxel value is the one
     * mo_df_build_ex stores. */
    const float* df_tree;      /* mo_df_tree_build output */
    float* df_lin;             /* float [N^3]: the voxel values computed so far */
    uint32_t* df_cells;        /* bit per cell ((N-1)^3): queued, then written */
    uint32_t* df_packets;      /* bit per 4x4x2 voxel packet: queued, then computed */
    int32_t* df_status;        /* bit 2: traversal stack overflow, 4: malformed tree, 8: queue full */
    int32_t* df_queue;         /* (pair index, cell) int32 pairs, df_queue_cap of them */
    int32_t* df_pqueue;        /* (pair index, packet) int32 pairs, 8 * df_queue_cap of them */
    int32_t* df_queue_count;   /* two counters per launch of the group */
    int32_t df_ntri;           /* target triangles */
    int32_t df_queue_cap;
    float df_band;             /* the build band (mo_df_loss_band(N)) */
    int32_t df_pad;
    /* Per-edge weights (CadEdgeLoss, src/interface/cad_layer.cc:152-223),
     * read only by mo_fused_step_weighted: mo_sell_fill_w's record-aligned
     * copy; NULL there means weight 1.  Each record contributes
     * (v1 - v0 - off) * w^2 to the gradient and ((v1 - v0 - off) * w)^2 to
     * the energy. */
    const float* sell_w;
} MoPair;

typedef struct MoTile {
    int32_t pair;    /* index into the MoPair array */
    int32_t slice0;  /* first 32-vertex slice of the tile */
    int32_t nslices; /* 1..8 slices (one warp each) */
    int32_t pad;
} MoTile;

/* One step (launch_index = 0.. within a group of launches; step t =
 * t0 + launch_index + 1).  tile_loss[(launch_index*max_tiles + tile)*8 + w]
 * gets the loss partial of warp w of the tile (MO_TILE_WARPS floats per
 * tile).  ntiles is read from device memory.  grid_ctas <= 0 picks a
 * persistent grid of resident CTAs. */
#define MO_TILE_WARPS 8
int mo_fused_step(const MoPair* pairs, const MoTile* tiles, const int32_t* ntiles, int max_tiles,
                  int launch_index, float* tile_loss, int grid_ctas, void* stream);
/* mo_fused_step for pairs with per-edge weights (MoPair.sell_w): the
 * CadLossFunction objective (src/python/layers/cad_loss_layer.py:9-31,
 * cad_layer.cc:79-223) -- 0.5 sum d^2 + w_edge * 0.5 sum |r * w_e|^2 -- and
 * its gradient in the serial-scatter order.  A separate instantiation, so
 * the unweighted kernel carries no weight loads. */
int mo_fused_step_weighted(const MoPair* pairs, const MoTile* tiles, const int32_t* ntiles, int max_tiles,
                           int launch_index, float* tile_loss, int grid_ctas, void* stream);
/* mo_fused_step for pairs with on-demand grids (df_cells set): also queues
 * the cells the step moves vertices into (see MoPair). */
int mo_fused_step_on_demand(const MoPair* pairs, const MoTile* tiles, const int32_t* ntiles, int max_tiles,
                            int launch_index, float* tile_loss, int grid_ctas, void* stream);
/* pair_loss[k*npairs + p] (double) = sum, in a fixed order, of the tile
 * partials of pair p (its MoPair tile0/ntiles range) for launches
 * k = 0..nlaunch-1: the layer loss 0.5*sum d^2 + w_edge*0.5*sum |r|^2 at the
 * positions before step t0+k+1. */
int mo_pair_loss(const MoPair* pairs, int npairs, int max_tiles, int nlaunch, const float* tile_loss,
                 double* pair_loss, void* stream);
/* On-demand distance field.  mo_df_lazy_bytes(N): the two bit sets of a
 * pair (cells, then packets; zero them before first use).  mo_df_lazy_seed
 * queues the cells of nv float4 positions (pair index `pair` of `pairs`)
 * and their packets, as a step does: cells into queue (cap entries),
 * packets into pqueue (8 * cap entries), counts[0] / counts[1] counting
 * them.  mo_df_lazy_fill computes the queued packets, then writes the
 * queued cells, and adds the two counts to totals[0..1] (device int64,
 * optional).  Both read the pair table from device memory.  Grids up to
 * MO_DF_LAZY_MAX_N per axis (df_status bit 16 above it). */
#define MO_DF_LAZY_MAX_N 1024
size_t mo_df_lazy_bytes(int N);
int mo_df_lazy_seed(const MoPair* pairs, int pair, const float* pos4, int64_t nv, int32_t* queue,
                    int32_t* pqueue, int32_t* counts, int cap, void* stream);
int mo_df_lazy_fill(const MoPair* pairs, const int32_t* queue, const int32_t* pqueue, const int32_t* counts,
                    int cap, int64_t* totals, void* stream);

/* ------------------------------------------------------------------------
 * Serving pool: admit / step / retire deformation requests.  A request is one
 * run of the reference's rigid_deform loop (src/python/rigid_deform.py:25-44:
 * InitializeDeformTemplate, NormalizeByTemplate, StoreRigidityInformation,
 * `steps` Adam steps of RigidLossFunction, Finalize) on its own source and
 * target.  The pool admits requests FIFO against an HBM byte budget, builds
 * each on one of its build streams (copies, DF build, CSR, sliced-ELL records;
 * memory from a stream-ordered pool), steps every active pair with one
 * replay of a captured CUDA graph of group_steps mo_fused_step launches per
 * mo_pool_progress call, and retires a pair (denormalised result in device
 * memory, final loss) right after the group in which its last step ran.  A
 * result is bit-identical whether its request ran alone or in any mix.
 * A pool is driven by one host thread; it has its own non-blocking streams.
 * No counterpart in the reference (its loop is one pair, synchronous).
 * ------------------------------------------------------------------------ */
typedef struct MoPool MoPool;

typedef struct MoPoolConfig {
    uint64_t hbm_budget_bytes; /* 0: 60% of the device's free memory at creation */
    int32_t max_pairs;         /* requests building, active or retiring at once */
    int32_t max_tiles;         /* tiles (<= 8 slices of 32 vertices) stepped at once */
    int32_t group_steps;       /* optimiser steps per group (one graph replay) */
    int32_t use_graph;         /* capture the group as a CUDA graph */
    int32_t max_building;      /* requests in their build phases at once (0: 8) */
    int32_t build_streams;     /* 0: 2 */
    int32_t layout;            /* default grid layout (MO_LAYOUT_*) */
    int32_t slices_per_tile;   /* default tile width, 1..8 (0: 8) */
    int32_t step_grid;         /* CTAs per fused-step launch (0: every resident CTA); fewer
                                * leave room on the SMs for concurrent DF builds */
    int32_t df_mode;           /* MO_DF_FULL: build every grid cell at admission;
                                * MO_DF_ON_DEMAND: build the traversal tree at admission and
                                * each cell when a vertex first reaches it (same values) */
} MoPoolConfig;
#define MO_DF_FULL 0
#define MO_DF_ON_DEMAND 1

typedef struct MoRequest {
    const float* srcV;   /* [nv,3] raw source vertices */
    const int32_t* srcF; /* [nf,3] source faces (the rigidity edges) */
    const float* tarV;   /* [ntv,3] raw target vertices */
    const int32_t* tarF; /* [ntf,3] target faces */
    int64_t nv, nf, ntv, ntf;
    int32_t inputs_on_host; /* the four arrays are host memory (else device) */
    int32_t N;              /* grid resolution */
    int32_t steps;          /* Adam steps */
    float w_edge;           /* edge-loss weight (lambda^2 of the rigid CLI) */
    double lr;              /* Adam learning rate (betas 0.9/0.999, eps 1e-8) */
    int32_t layout;         /* -1: the pool's default */
    int32_t slices_per_tile;/* 0: the pool's default */
    int32_t df_method;      /* MO_DF_AUTO / BRUTE / LBVH */
    int32_t df_packet;      /* MO_PACKET_* */
    float df_band;          /* < 0: mo_df_loss_band(N); 0: exact grid; > 0: this band */
    int32_t out_on_host;    /* V_out is host memory (pinned, for the copy to overlap) */
    float* V_out;           /* optional [nv,3]: the denormalised result, written at retirement */
    float* V_normalized_out;/* optional device [nv,3]: the result in the target-normalised frame */
} MoRequest;

#define MO_REQ_FAILED (-1)
#define MO_REQ_QUEUED 0
#define MO_REQ_BUILDING 1
#define MO_REQ_ACTIVE 2
#define MO_REQ_DONE 3

typedef struct MoPoolStats {
    int64_t submitted, done, failed;
    int64_t groups;         /* group replays issued */
    int64_t fused_launches; /* mo_fused_step launches issued (captured ones counted per replay) */
    uint64_t bytes_in_use;  /* admission estimate of the requests holding memory */
    uint64_t peak_bytes;
    int32_t queued, building, active, retiring;
    int32_t active_tiles;
    int32_t fill_launches_per_step; /* kernels of the on-demand fill after each fused step (0: full grids) */
} MoPoolStats;

int mo_pool_create(const MoPoolConfig* cfg, MoPool** pool_out);
int mo_pool_destroy(MoPool* pool);
/* Queue a request.  The input arrays must stay valid and unchanged until the
 * request is finished (DONE or FAILED), and so must the optional output
 * arrays, which the pool fills on its step stream as the request retires
 * (complete once the request is DONE).  Checks sizes and options on the
 * host; invalid meshes (a face index out of range) fail the request later. */
int mo_pool_submit(MoPool* pool, const MoRequest* req, int64_t* id_out);
/* Admit, advance builds, run one group over the active pairs, collect
 * retirements.  block != 0: when nothing is active, wait for the oldest build
 * or retirement before returning.  n_finished_out: requests DONE or FAILED so far. */
int mo_pool_progress(MoPool* pool, int block, int64_t* n_finished_out);
/* Progress until every submitted request is finished (or, on hold, built). */
int mo_pool_wait(MoPool* pool);
/* Pop up to max_ids ids of requests finished since the last call, in order. */
int mo_pool_completed(MoPool* pool, int64_t* ids, int max_ids, int* n_out);
int mo_pool_state(MoPool* pool, int64_t id, int32_t* state_out);
/* The failure message of a FAILED request (empty otherwise). */
int mo_pool_error(MoPool* pool, int64_t id, char* buf, size_t buf_bytes);
/* Copy a DONE request's fitted vertices [nv,3]: V_out denormalised (as
 * Finalize returns them), V_normalized_out in the target-normalised frame;
 * either may be NULL; host or device memory per out_on_host.  loss_out
 * (host, optional): the layer loss evaluated in the last step.  Synchronous. */
int mo_pool_result(MoPool* pool, int64_t id, float* V_out, float* V_normalized_out, int out_on_host,
                   double* loss_out);
/* Forget a finished request and recycle its result memory. */
int mo_pool_release(MoPool* pool, int64_t id);
/* hold != 0: progress admits and builds but does not step (steady-state
 * measurements: build everything, then mo_pool_run_groups). */
int mo_pool_set_hold(MoPool* pool, int hold);
/* Record CUDA events around each group for mo_pool_group_time. */
int mo_pool_set_timing(MoPool* pool, int enable);
/* Run `groups` groups over the active pairs now (ignores hold). */
int mo_pool_run_groups(MoPool* pool, int groups);
/* Total device time (ms) of the timed groups since the last call and their
 * algorithmic bytes (104 per vertex + 44 per half-edge per pair-step). */
int mo_pool_group_time(MoPool* pool, double* ms_out, double* bytes_out);
int mo_pool_stats(MoPool* pool, MoPoolStats* out);
/* On-demand mode: cells written and voxel packets computed so far, over all
 * requests (out2[0], out2[1]); zeros for full grids.  Synchronises the
 * pool's streams. */
int mo_pool_fill_totals(MoPool* pool, int64_t* out2);
/* Return freed device memory the pool keeps for reuse to the device, down to
 * keep_bytes (synchronises the pool's streams). */
int mo_pool_trim(MoPool* pool, uint64_t keep_bytes);
/* The pool's step stream (a cudaStream_t). */
int mo_pool_step_stream(MoPool* pool, void** stream_out);
/* ------------------------------------------------------------------------
 * Reverse (target -> source) nearest-point loss.  Replaces ReverseLossLayer
 * (src/python/layers/reverse_loss_layer.py:14-25): ii = cKDTree(src_V)
 * .query(tar_V, k=1); loss = 0.5 * sum |src_V[ii] - tar_V|^2, and its
 * autograd backward.  Used per step by inverse_deform.py:26-31 and
 * cad_deform2.py:46-52.
 * ------------------------------------------------------------------------ */
size_t mo_nn_scratch_bytes(int64_t np, int64_t nq);
/* idx_out[q] (int32 [nq]) = the index of the point of P [np,3] nearest to
 * Q[q] (squared Euclidean distance in double, summed x, y, z, as cKDTree
 * computes it from float32 input; exact ties go to the lowest index);
 * d2_out (optional, double [nq]) = that squared distance.  scratch NULL:
 * allocated stream-ordered.  Synchronises `stream`; MO_ERR_DEVICE when a
 * query is not finite or no point is. */
int mo_nn_query(const float* P, int64_t np, const float* Q, int64_t nq, int32_t* idx_out, double* d2_out,
                void* scratch, size_t scratch_bytes, void* stream);
size_t mo_reverse_loss_scratch_bytes(int64_t ns, int64_t nt);
/* loss_out (device double [1]) = 0.5 * sum over t of |src[idx[t]] - tar[t]|^2,
 * the differences and squares in float like the reference's tensors, summed
 * in double in a fixed order.  status_out: optional device int32; when given
 * the call does not synchronise and bit 0 is OR-ed in for an index outside
 * [0, ns) (that term skipped); when NULL the call synchronises and returns
 * MO_ERR_DEVICE for it. */
int mo_reverse_loss_forward(const float* src, int64_t ns, const float* tar, int64_t nt, const int32_t* idx,
                            double* loss_out, void* scratch, size_t scratch_bytes, int32_t* status_out,
                            void* stream);
/* grad_src [ns,3] = the gradient of grad_out (device float [1]) * that loss
 * with respect to src, bit-identical to torch's CPU autograd of the
 * reference expression: per source vertex, over its matched targets in
 * increasing t, the sum from zero of (g*l + g*l), l = src[i] - tar[t],
 * g = 0.5 * grad_out.  status_out as above. */
int mo_reverse_loss_backward(const float* src, int64_t ns, const float* tar, int64_t nt, const int32_t* idx,
                             const float* grad_out, float* grad_src, void* scratch, size_t scratch_bytes,
                             int32_t* status_out, void* stream);

/* ------------------------------------------------------------------------
 * Sparse linear propagation.  Replaces SolveLinear (src/interface/
 * linear_layer.cc:5-79): LinearEstimation (src/lib/linear.cc:10-112; with_rot
 * 0) and LinearEstimationWithRot (linear.cc:114-230; with_rot 1), in place
 * on V (float [nv,3], read and written like the reference's tensor).  The
 * reference factorises the assembled system with SimplicialLDLT; here it is
 * solved matrix-free by Jacobi-preconditioned conjugate gradients in double,
 * from x0 = V, until every coordinate's relative residual is <= tol (or
 * max_iter iterations: MO_ERR_DEVICE).  with_rot 0: F [nf,3] and E [ne,2]
 * give the edge springs, ref [nv] the graph node of every vertex, G [ng,3]
 * the graph positions.  with_rot 1: F only (E, ref ignored), G [nv,3] the
 * per-vertex targets (ng == nv).  Synchronises `stream`.
 * ------------------------------------------------------------------------ */
size_t mo_solve_linear_scratch_bytes(int64_t nv, int64_t nf, int64_t ne, int64_t ng, int with_rot);
int mo_solve_linear(float* V, int64_t nv, const int32_t* F, int64_t nf, const int32_t* E, int64_t ne,
                    const int32_t* ref, const float* G, int64_t ng, double rigidity, int with_rot, double tol,
                    int max_iter, void* scratch, size_t scratch_bytes, int* iters_out, double* rel_residual_out,
                    void* stream);

/* ------------------------------------------------------------------------
 * Velocity-field ODE deformation (the NeuralODE variant,
 * src/python/layers/neuralode_fast.py:10-31,55-57; here an autonomous
 * 3 -> 256 -> 256 -> 256 -> 3 softplus MLP integrated by fixed-step RK4).
 * Fused FP32 kernels over 64-vertex tiles; a narrower MLP runs zero-padded
 * to mo_mlp_width().  Weights: W1 [M,3], b1 [M], W2 and W3 [M,M] (row =
 * output unit), b2, b3 [M], W4 [3,M], b4 [3], all row-major.
 * ------------------------------------------------------------------------ */
/* The kernels' hidden width M (256). */
int mo_mlp_width(void);
/* 64-vertex tiles of n rows (the grid of mo_mlp_fwd / mo_mlp_bwd). */
int64_t mo_mlp_tiles(int64_t n);
/* Floats in one partial row of mo_mlp_bwd (one row per warp, 8 per tile). */
int mo_mlp_partial_floats(void);
/* WT = W^T for an M x M matrix (the forward takes W2^T and W3^T). */
int mo_mlp_transpose(const float* W, float* WT, void* stream);
/* One MLP evaluation k = f(u) of n rows with its RK4 stage update:
 * unext = x + a*k (unext may be NULL), acc = (init_acc ? x : acc) + w*k.
 * store (may be NULL): Z1, H1, Z2, H2, Z3, H3 (pre- and post-softplus of the
 * three hidden layers, each [n,M]) at store + i*astride, for mo_mlp_bwd. */
int mo_mlp_fwd(const float* u, const float* x, int64_t n, const float* W1, const float* b1, const float* W2T,
               const float* b2, const float* W3T, const float* b3, const float* W4, const float* b4, float a,
               float w, int init_acc, float* unext, float* acc, float* store, int64_t astride, void* stream);
/* The vector-Jacobian product of one evaluation for dL/dk = gk [n,3], from
 * its stored activations: gu [n,3] = dL/du; gz3, gz2 [n,M] = dL/dZ3, dL/dZ2
 * (for mo_mlp_wgrad); partial gets one row of mo_mlp_partial_floats() per
 * warp (8 * mo_mlp_tiles(n) rows) holding that warp's dW4, db4, db3, db2,
 * db1, dW1 terms, for mo_mlp_partial_reduce. */
int mo_mlp_bwd(const float* gk, const float* u, int64_t n, const float* W1, const float* W2, const float* W3,
               const float* W4, const float* store, int64_t astride, float* gz3, float* gz2, float* gu,
               float* partial, void* stream);
/* dW4 [3,M], db4 [3], db3, db2, db1 [M], dW1 [M,3] += the sums of `rows`
 * partial rows (summed in groups of consecutive rows, then the groups in
 * order: deterministic).  scratch: mo_mlp_partial_reduce_bytes(). */
size_t mo_mlp_partial_reduce_bytes(void);
int mo_mlp_partial_reduce(const float* partial, int64_t rows, float* scratch, float* dW4, float* db4, float* db3,
                          float* db2, float* db1, float* dW1, void* stream);
/* dW [M,M] += A^T B (A, B [rows,M]: dW[o][i] = sum_r A[r][o] B[r][i]),
 * split over rows into `splits` partial sums (partial:
 * mo_mlp_wgrad_partial_bytes(splits)) added in split order. */
size_t mo_mlp_wgrad_partial_bytes(int splits);
int mo_mlp_wgrad(const float* A, const float* B, int64_t rows, int splits, float* partial, float* dW,
                 void* stream);

/* sizeof(MoPair) and sizeof(MoTile) as compiled (host pointers), so that
 * bindings in other languages can check their struct layout. */
int mo_abi_sizes(size_t* pair_bytes, size_t* tile_bytes);
/* float [n,3] <-> float4 [n] position packing. */
int mo_pack_pos(const float* V, int64_t n, float* pos4, void* stream);
int mo_unpack_pos(const float* pos4, int64_t n, float* V, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MESHODE_GB300_H_ */
