/*
 * C ABI of the GB300 (sm_103a) mesh-surface DEM timestep engine.
 *
 * Library: sand_atlas_dem_gb300/_lib/libsanddem_gb300.so (built by
 * sand_atlas_dem_gb300.native.build()).  Plain pointers and sizes only; all
 * buffer pointers are CUDA device pointers, `stream` is a cudaStream_t (or
 * NULL for the legacy default stream, which graph capture does not accept).
 *
 * Buffer block (SDG_BUFFER_COUNT pointers, `bytes` their sizes):
 *   [0, 77)   the reference Resources fields in declaration order
 *             (src/sand_atlas_dem/shaders/solver.slang:20-100) — the same
 *             order the reference CPU backend binds in its generated
 *             cpu_dispatch (src/sand_atlas_dem/cpu.py:189-300);
 *   [77, 136) this backend's extension buffers, in the order of
 *             sand_atlas_dem_gb300.engine.EXTENSION_ORDER (leaf tables,
 *             node ranks, pair-by-second-grain runs, directed-pair branches,
 *             leaf masks, (directed pair, leaf) items and hit masks, contact
 *             pair ids, the written and committed history pair tables, work
 *             counters, scan partials, the per-survivor hit scratch, the
 *             survivor count of each item, per directed pair the target
 *             enclosure plane facing the source, the specimen of each
 *             grain and each specimen's bin grid, the learned culler's
 *             per-shape FP32 parameters, BF16 hidden weights, margins and
 *             two counters, the survivor mask and first survivor of each
 *             item and the (item, node slot) list of survivors -- the nodes
 *             left for the exact query after the conservative filters --
 *             and, for the learned culler, a keep flag per survivor, its
 *             exclusive scan and the list of kept survivors, and per
 *             directed pair the enclosure plane carried into the source
 *             grain's frame with its rejection-bound terms, and the
 *             triangle BVH as one record per node with both children's
 *             bounds, and per shape a 48^3 grid of certified lower bounds of
 *             the signed distance with its origin and cell size, and the
 *             triangle nearest to each cell centre, and the pose the stored
 *             node-filter results were built at: each grain's orientation,
 *             each pair's branch and the pair list itself, and the walk
 *             order of the stored exact-query list: each kept survivor's
 *             bucket (target shape, coarse cell), and the count and first
 *             slot of each bucket, and for the SDF geometry each pair's
 *             contact counts per virtual lane of the reference's 64-lane
 *             group, 32 words per pair, and per stored walk-list slot its
 *             nearest-triangle certificate: the point it was taken at with
 *             the distance gap, and the triangle with a tying triangle of
 *             another leaf (two words; or a dormant mark), and with planes the
 *             plane-contact count of each (wall, grain), wall-major, its
 *             exclusive scan, and the first contact of each (wall, grain)
 *             on the side being written and on the committed side, and per
 *             stored walk-list slot its node record -- source grain, target
 *             grain, directed pair and packed sample index -- and its
 *             (item, node slot)).
 * Value block (SDG_VALUE_COUNT doubles): the 25 reference Config scalars in
 * declaration order (solver.slang:12-19, normalized units as
 * src/sand_atlas_dem/gpu.py:490-518 builds them), then leaf mask words per
 * directed pair, (directed pair, leaf) item capacity, a flag that fuses
 * captureContactKinematics into beginStep, and the number of independent
 * periodic specimens batched in the buffers (cell rows 3 per specimen,
 * cellLog and referenceCell rows 2 per specimen; 1 = the reference case),
 * whether the learned culler runs in front of the exact node query, six
 * launch shapes chosen by the autotuner (0 = default): node-filter CTAs per
 * SM, node-filter warps per CTA (4 or 8), pair set-up/leaf-cull CTAs per SM,
 * contact emit/law CTAs per SM, gather warps per SM and exact-query CTAs per
 * SM (launch shapes never change results), the survivor capacity (nodes
 * left for the exact query per step; overflow raises the contact-capacity
 * flag), whether nodes the distance-bound grid certifies outside their
 * target skip the exact query, and the filter margin: the reach, in the
 * target shape's unscaled frame, by which the leaf cull and node filter grow
 * their tests when they store their results; the results are reused while
 * no grain has moved that far relative to a partner (0 = run the filters
 * every step; contacts are identical either way).
 *
 * Return codes: 0 success; 1 argument error; 2 CUDA error.  The message of
 * the last error on the calling thread is sdg_last_error().  Solver failures
 * (capacity, penetration, nonfinite state, ...) are not return codes: they
 * are the bit flags of control[0] with the reference meanings
 * (src/sand_atlas_dem/gpu.py:11-26), read back by the host after a chunk.
 */
#ifndef SAND_DEM_GB300_H
#define SAND_DEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SDG_BUFFER_COUNT 136
#define SDG_VALUE_COUNT 39
#define SDG_PHASES 9

/* ABI revision of this header. */
int sdg_abi_version(void);
/* SDG_BUFFER_COUNT and SDG_VALUE_COUNT as compiled into the library. */
int sdg_buffer_count(void);
int sdg_value_count(void);
/* Text of the last nonzero return on this thread. */
const char* sdg_last_error(void);

/*
 * Launches one reference-named kernel or step phase on `stream`.
 * Replaces the reference's per-kernel `cpu_dispatch(count, buffers, bytes,
 * values)` of src/sand_atlas_dem/cpu.py:303-428 (NativeKernel.dispatch) and
 * the Metal adapter's `dispatch(name, n, encoder, r=bindings)` of
 * src/sand_atlas_dem/backend.py:9-121.  Names: beginStep, advanceCell,
 * checkRebuild, finishStep, captureContactKinematics, checkContactTimestep,
 * diagnosticRows, fabricRows, neighbours (clearBins..emitPairs + Scan),
 * collect (resetMeshContacts, prepareMeshPairs, collectMeshFrontiers,
 * collectWallContacts), collectCull / collectQuery / collectEmit /
 * collectWalls (its parts), resolveContacts (friction history + contact
 * law, grain and plane contacts), gather, gatherWallRows, advanceWalls,
 * refreshWallPower (solver.slang:669-687, :834-856, :950-955), and the
 * sequences forces / forcesNoCapture (Engine.forces, gpu.py:547-565) and
 * step (Engine._advance_once body, gpu.py:714-724).  `count` is the thread
 * count of per-element kernels (N grains, pairCapacity, ...).
 */
int sdg_dispatch(const char* kernel, uint32_t count, void* const* buffers, const uint64_t* bytes,
                 const double* values, uint32_t nvalues, void* stream);

/*
 * 256-wide binary tree reduction of `rows` float4 rows per element, summing
 * (row `max_row`, component w: maximum), one output row set per 256 inputs.
 * Replaces the reference's reduceRows / reduceFabric
 * (src/sand_atlas_dem/shaders/diagnostic.slang:3-28) used by
 * Engine.diagnostics (gpu.py:746-891); `max_row` = -1 for none.
 */
int sdg_reduce_rows(const void* input, void* output, uint32_t n, uint32_t rows, int32_t max_row,
                    void* stream);

/*
 * One level of the per-wall reduction of the (wall, grain) rows (reaction |
 * contact count, moment | power, work; 3 float4 per row, wall-major, n rows
 * per wall): output holds ceil(n / 256) row sets per wall, the count summed
 * as an integer.  Replaces the reference's reduceWallRows
 * (src/sand_atlas_dem/shaders/diagnostic.slang:33-49) of Engine.diagnostics
 * (gpu.py:774-786).
 */
int sdg_reduce_wall_rows(const void* input, void* output, uint32_t n, uint32_t walls, void* stream);

/*
 * Device-wide exclusive scan of n uint32 values: out[i] = in[0] + ... +
 * in[i-1]; *total (device pointer, may be NULL) receives the sum.  Replaces
 * the reference's hierarchical Scan (src/sand_atlas_dem/gpu.py:65-91,
 * shaders/scan.slang:1-28: blockScan + addBlocks).  `partials` is caller-
 * owned device scratch of sdg_scan_partials() uint32 words.
 */
int sdg_exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* total, uint32_t* partials,
                       void* stream);
int sdg_scan_partials(void);

/*
 * Device-to-device copies of n buffers on `stream` (dst[k] <- src[k],
 * bytes[k] each, one cudaMemcpyAsync per buffer).  The transactional backup
 * of a chunk and its restore, which the reference does with encoder buffer
 * copies (src/sand_atlas_dem/gpu.py:729-743, backend.py copy_buffer).
 */
int sdg_copy_buffers(void* const* dst, void* const* src, const uint64_t* bytes, uint32_t n, void* stream);

/*
 * The same scan with its block partials in a fixed array of this library
 * (4,864 bytes per device) instead of caller scratch; it allocates nothing.
 * No counterpart in the reference: it serves callers that hold only the
 * buffers they were handed and no device allocator (a cgo, JNI or ctypes
 * stub), or whose device-memory budget is fixed after set-up.  The first call
 * on a device, with that device current, looks the array up; it must come
 * before any stream capture on that device.  A device reset replaces the
 * context, and the first call after it looks the array up again (the same
 * rule applies to that call).  n above SDG_SCAN_STATIC_MAX_N is rejected
 * (returns 1, text in sdg_last_error); so is a call made while an earlier,
 * unrelated CUDA error is pending (it is reported, not cleared, and nothing
 * is launched).  Nothing needs zeroing beforehand.  Calls in flight at the
 * same time on one device share the array and race: issue them on one stream.
 */
#define SDG_SCAN_STATIC_MAX_N (1u << 30)
int sdg_exclusive_scan_static(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* total, void* stream);

/*
 * Engine handle holding the captured CUDA graphs of one step for each
 * history-side orientation.  Replaces the per-chunk command encoder of
 * Engine._advance_once (gpu.py:672-744): one graph launch per step.
 */
void* sdg_engine_create(void);
void sdg_engine_destroy(void* engine);

/*
 * Advances `steps` timesteps starting from the history side the buffers
 * describe (meta/slip/normalArea/... = side written first), alternating
 * sides every step as gpu.py:725 does.  use_graph != 0 replays captured
 * graphs (recaptured when buffers or values change).  No host
 * synchronization; solver flags accumulate in control[0].
 */
int sdg_engine_advance(void* engine, void* const* buffers, const uint64_t* bytes, const double* values,
                       uint32_t nvalues, uint32_t steps, uint32_t use_graph, void* stream);

/*
 * Engine.diagnostics (src/sand_atlas_dem/gpu.py:746-891) in one call: the
 * diagnostic rows (solver.slang:922-947) and fabric rows with their 256-wide
 * tree reductions (diagnostic.slang:3-28) through two device scratch buffers
 * of scratch_bytes each (at least ceil(max(N, pairCapacity) / 256) x 8 rows x
 * 16 bytes), then 272 bytes copied to `host` (pinned): the 8 reduced
 * diagnostic rows, the 2 reduced fabric rows, the first 3 cell rows and the
 * 16 control words.  The caller waits on the stream before reading `host`.
 * Replaces the reference's per-reduction dispatches and reads.
 */
int sdg_engine_diagnostics(void* const* buffers, const uint64_t* bytes, const double* values, uint32_t nvalues,
                           void* scratch_a, void* scratch_b, uint64_t scratch_bytes, void* host, void* stream);

/*
 * One committed step with CUDA events between phases; writes SDG_PHASES
 * device milliseconds: drift, neighbours, pair cull, node filter (with the
 * survivor list and the learned culler), exact node queries, contact emit,
 * friction history + contact law, force gather, final kick.
 * Replaces Engine.profile_step's timestamp queries (gpu.py:938-1014).
 */
int sdg_engine_profile(void* engine, void* const* buffers, const uint64_t* bytes, const double* values,
                       uint32_t nvalues, float* phase_ms, void* stream);

/*
 * Learned culler (no reference counterpart): per-shape networks
 * h0 = sin(W0 p + b0), h1 = relu(W1 h0 + b1), y = w2.h1 + b2 (64 wide)
 * trained on exact signed distances.  sdg_culler_param_count() floats per
 * shape.  sample: shell candidates labelled by the exact BVH distance;
 * compact: keep accepted candidates in index order; train_step: one Adam
 * step on every shape (forward/backward kernels; squared error with an
 * over-prediction at an inside point weighted by `over`); gradients: forward
 * and backward only; round: BF16 hidden weights for inference; eval: FP32
 * evaluation with BF16 hidden weights; tile_eval: the run-time tensor-core
 * evaluation (tcgen05, 128-point tiles; NaN where a tensor-core wait gave
 * up); inside_max: per-shape largest prediction at inside points
 * (the calibrated margin, as an ordered integer); surface: points on each
 * shape's surface (shape s owns packed triangles [tri_start[s],
 * tri_start[s+1])), label 0, for the margin's boundary term.
 */
int sdg_culler_param_count(void);
int sdg_culler_sample(void* const* buffers, const uint64_t* bytes, const double* values, uint32_t nvalues,
                      uint32_t shapes, uint32_t count, uint32_t seed, float shell, uint32_t inside_only,
                      void* out_points, void* accept, void* stream);
int sdg_culler_surface(const void* triangles, const void* tri_start, uint32_t shapes, uint32_t count, uint32_t seed,
                       void* out_points, void* stream);
int sdg_culler_compact(const void* points, const void* accept, const void* offsets, uint32_t shapes,
                       uint32_t count, uint32_t capacity, void* out, void* stream);
int sdg_culler_train_step(void* params, const void* points, uint32_t shapes, uint32_t points_per_shape,
                          uint32_t batch, uint32_t step, uint32_t seed, float scale, float over, float lr,
                          void* grads, void* m, void* v, void* scratch, float* loss_out, void* stream);
int sdg_culler_gradients(const void* params, const void* points, uint32_t shapes, uint32_t points_per_shape,
                         uint32_t batch, uint32_t step, uint32_t seed, float scale, float over, void* grads,
                         void* scratch, void* stream);
int sdg_culler_round(const void* params, void* w1_bf16, uint32_t shapes, void* stream);
int sdg_culler_eval(const void* params, const void* w1_bf16, const void* points, uint32_t shapes, uint32_t count,
                    void* out, void* stream);
int sdg_culler_tile_eval(const void* params, const void* w1_bf16, const void* points, uint32_t shapes,
                         uint32_t count, void* out, void* stream);
int sdg_culler_inside_max(const void* points, const void* predictions, uint32_t shapes, uint32_t count,
                          void* keys, void* stream);
/* Cells per shape of the culler's margin grid (8^3 over the shape's root
 * box); the engine's cullerMargin buffer holds per shape the whole-shape
 * margin then one margin per cell.  inside_max_cells: per (shape, cell) the
 * ordered-integer maximum prediction at inside points and their count. */
int sdg_culler_margin_cells(void);
int sdg_culler_inside_max_cells(const void* points, const void* predictions, uint32_t shapes, uint32_t count,
                                const void* roots, const void* mesh_min, const void* mesh_max, void* keys,
                                void* counts, void* stream);

/*
 * Kernel launches of a captured step that skips both conditional bodies (0
 * before the first capture).  The captured step holds the neighbour build
 * and, with stored filter results, the filter build as conditional-node
 * bodies keyed on device flags (the reference re-encodes the rebuild
 * dispatches every step and lets them exit early, gpu.py:547-565).
 */
int sdg_engine_kernels_per_step(void* engine);
/*
 * Kernel launches inside conditional body `branch` of a captured step: 0 =
 * the neighbour build (steps whose rebuild flag is set), 1 = the filter build
 * (steps that build the stored filter results).  -1 for a bad argument.
 */
int sdg_engine_branch_kernels(void* engine, int branch);

/*
 * The two median-split trees of the packed mesh layout, built on the device
 * for every shape at once.  Replaces the host recursions of the reference's
 * mesh.pack_meshes (src/sand_atlas_dem/mesh.py:33-56, the source-node
 * cluster tree, leaf = 64; mesh.py:164-201, the triangle BVH, leaf = 4),
 * whose results it reproduces bit for bit.
 *
 * Items of shape s are counts[s] consecutive rows of `keys` (float x, y, z,
 * unused; finite), the split coordinates: sample points, or triangle centres
 * (mean of the three FP32 vertices, as the reference computes it).  `low` and
 * `high` (same layout) are each item's box, whose union bounds a node (the
 * triangles' vertex minimum and maximum); both null: the box is the point.
 * `counts` is a HOST array of `shapes` nonzero counts, at most 2^30 items in
 * all.  Outputs, in preorder with the shapes one after another: `order` (one
 * word per item position: the row, within its shape, of the item placed
 * there; leaves in preorder),
 * `records` (4 words per node: escape = index past the node's subtree, first
 * position and count for a leaf or 0, 0 for an internal node, depth) and
 * `node_low`/`node_high` (4 floats per node: the bounds moved one ulp
 * outward, then 0).  Nodes of shape s: sdg_median_tree_nodes(counts[s],
 * leaf).  Scratch: sdg_median_trees_scratch(counts, shapes, leaf) bytes of
 * device memory.  The call returns when the trees are built (it waits on
 * `stream`).  Return codes as above.
 */
uint32_t sdg_median_tree_nodes(uint32_t items, uint32_t leaf);
uint64_t sdg_median_trees_scratch(const uint32_t* counts, uint32_t shapes, uint32_t leaf);
int sdg_median_trees(const float* keys, const float* low, const float* high, const uint32_t* counts, uint32_t shapes,
                     uint32_t leaf, uint32_t* order, uint32_t* records, float* node_low, float* node_high,
                     void* scratch, uint64_t scratch_bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SAND_DEM_GB300_H */
