/*
 * tb.h -- C ABI of the GB300 tropical contraction engine.
 *
 * This is the drop-in boundary for the hot path of TensorBranching.jl's
 * dynamic_ob_mis: the tropical (max,+) contraction of the independent-set
 * tensor network of every slice / branch, plus "+ r" and the max over slices.
 *
 * Reference interfaces it replaces (paths inside the TensorBranching.jl tree):
 *   solve_slice(branch, element_type, usecuda)::T      src/dynamic_ob.jl:30-34
 *     GenericTensorNetwork(IndependentSet(g, w), uncompress(code), Dict())
 *     solve(net, SizeMax(), T = element_type, usecuda)  src/dynamic_ob.jl:31-32
 *   contract_slices(branches, element_type, usecuda)    src/dynamic_ob.jl:36-48
 *   maximum(res)                                        src/dynamic_ob.jl:27
 *   CompressedEinsum{ixs, iy, ct} / uncompress          src/types.jl:51-79
 *   SlicedBranch{p, code, r}                            src/types.jl:85-103
 *
 * Conventions.  Labels are dense ids 0..n_labels-1 (a Julia caller passes
 * vertex v as v-1).  Every label has dimension 2.  Tensors are column-major:
 * the first label of a tensor is its fastest index.  A network is given as
 * its leaf tensors (ixs), its open labels (iy; empty for the MIS scalar) and a
 * binary contraction tree in post-order pairs: internal node j has children
 * children[2j], children[2j+1]; ids < n_tensors are leaves, id n_tensors + k
 * is internal node k < j; the last internal node is the root.
 *
 * Tensor contents for the MIS path (GenericTensorNetworks IndependentSet):
 * a leaf with one label v is the vertex tensor [0, w_v]; a leaf with two
 * labels is the edge tensor [[0,0],[0,-inf]] (a self-loop [v,v] is its
 * diagonal [0,-inf]).
 *
 * Errors.  Every entry point returns tb_status; no C++ exception crosses the
 * ABI.  tb_last_error(ctx) returns a message for the last failure on that
 * context (thread-local to the calling thread).  A context is used by one
 * host thread at a time, except the streaming calls tb_submit / tb_poll /
 * tb_wait, which may be called from any thread.  Plans are immutable after
 * tb_plan_bind_mis and may be shared between calls.
 *
 * Memory.  The library copies every input array; callers keep ownership of
 * what they pass.  Output arrays are host memory written before return.
 */
#ifndef TB_H
#define TB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t tb_status;
#define TB_OK 0
#define TB_ERR_INVALID 1     /* malformed plan or argument */
#define TB_ERR_OOM 2         /* device memory budget exceeded */
#define TB_ERR_TIMEOUT 3     /* a bounded device-side wait ran out */
#define TB_ERR_CUDA 4        /* a CUDA runtime call failed */
#define TB_ERR_UNSUPPORTED 5 /* valid request outside this build's limits */
#define TB_ERR_BUSY 6        /* streaming queue full */

#define TB_DTYPE_F32 0 /* Tropical{Float32}: -inf is the additive zero */
#define TB_DTYPE_I32 1 /* int32 with sentinel TB_I32_NEG standing for -inf */
#define TB_I32_NEG (-536870912)

/* Execution modes of tb_solve_batch. */
#define TB_MODE_PLAIN 0   /* drop-in: one item at a time, per-contraction launches
                             (permute + batched tropical GEMM + permute), result
                             copied back after each item, as the reference's loop */
#define TB_MODE_BATCHED 1 /* every item in one persistent launch over a device
                             work queue, replayed from a captured CUDA graph */
#define TB_MODE_LAYERED 2 /* fused per-contraction launches over all items,
                             captured in a CUDA graph */
#define TB_MODE_AUTO 3    /* the schedule tb_autotune chose for this context
                             (tuned on first use when tb_options.autotune is 1;
                             TB_MODE_BATCHED before any tuning) */
#define TB_MODE_FUSED 4   /* one block per item contracts the whole network in
                             shared memory, one launch for the batch; every
                             plan must have the small form (tensors of at most
                             2^13 entries, at most 48 KiB live per network,
                             tb_plan_stats.small_words > 0), else
                             TB_ERR_UNSUPPORTED */

typedef struct tb_ctx tb_ctx;
typedef struct tb_plan tb_plan;

typedef struct tb_options {
  int32_t dtype;            /* TB_DTYPE_* */
  int32_t use_graphs;       /* 1: capture batched launches in CUDA graphs */
  int64_t max_device_bytes; /* arena budget; 0 = 80% of free memory at create */
  int32_t timeout_ms;       /* bound on every device-side wait (default 20000) */
  int32_t autotune;         /* 1: the first TB_MODE_AUTO solve runs tb_autotune */
  int32_t persistent_ctas;  /* CTAs of the persistent executor; 0 = 2 per SM */
  int32_t gemm_i16;         /* 0 (default): every contraction computes in the
                               context's dtype.  1 (TB_DTYPE_F32 only): GEMM tiles
                               of a plan whose bound weights are integers >= 0
                               summing below 8192 compute in packed int16 pairs
                               (exact for such values: same results, twice the
                               SIMT rate); other plans stay f32 */
  int32_t reserved[8];
} tb_options;

typedef struct tb_plan_stats {
  double tc;              /* log2 sum over nodes of 2^|labels(node)| */
  double sc;              /* log2 of the largest tensor */
  double rwc;             /* log2 of total elements read + written */
  double ops;             /* algorithmic tropical ops per item: 2 per (max,+) pair */
  double bytes;           /* algorithmic bytes per item: 4 (|A|+|B|+|C|) per node */
  int64_t arena_bytes;    /* device bytes one item of this plan occupies */
  int32_t n_steps;        /* compiled contraction steps */
  int32_t n_tensors;
  int32_t n_open;         /* labels left open in the root tensor */
  int32_t n_sliced;       /* labels fixed per item by tb_solve_batch */
  int32_t n_tiles;        /* CTA tiles of one item in the fused form */
  int32_t small_words;    /* shared-memory words of the TB_MODE_FUSED form (0: none) */
  int32_t reserved[6];
} tb_plan_stats;

/* Result of tb_autotune: the chosen tile size and schedule. */
typedef struct tb_tune_result {
  int32_t mode;        /* TB_MODE_BATCHED, TB_MODE_LAYERED or TB_MODE_FUSED */
  int32_t tile_bits;   /* stream tiles of up to 2^tile_bits outputs (8..11) */
  int32_t ctas_per_sm; /* resident CTAs per SM of the persistent executor */
  int32_t chunk_div;   /* runs of stream tiles hold >= 1/(chunk_div CTAs) of a level */
  double ms;           /* device time of the batch with the chosen settings */
  double ms_default;   /* device time with the defaults */
  int32_t n_tried;     /* configurations timed */
  int32_t stream_ctas_per_sm; /* resident CTAs per SM of the per-level stream kernel:
                                 3 (80 registers a thread) or 2 (128) */
  int32_t kpart_atomic; /* 1: split-K GEMM parts combine by atomic max into the
                           output (items whose values are all >= 0 or -inf);
                           0: through partials and a max step */
  int32_t reserved[5];
} tb_tune_result;

/* Fill *opt with defaults (f32, graphs on, autotune on for TB_MODE_AUTO). */
void tb_options_default(tb_options* opt);

/* Create / destroy a context bound to CUDA device `device`. */
tb_status tb_ctx_create(int32_t device, const tb_options* opt, tb_ctx** out);
/* Plans created on ctx may still be passed to tb_plan_destroy afterwards
 * (and to nothing else). */
void tb_ctx_destroy(tb_ctx* ctx);
const char* tb_last_error(const tb_ctx* ctx);
/* Library version string, e.g. "tb 0.1 sm_103a". */
const char* tb_version(void);

/*
 * Compile a contraction plan.
 *   ixs       : n_tensors leaf label lists, CSR (ix_off[n_tensors+1], ix_lab)
 *   iy        : n_iy open labels of the result (empty for the MIS value)
 *   children  : n_nodes = n_tensors - 1 post-order pairs (see above)
 *   node_iy   : optional explicit output labels of every internal node (CSR
 *               node_iy_off[n_nodes+1], node_iy_lab), e.g. the eins.iy of each
 *               node of an OMEinsum DynamicNestedEinsum; NULL derives them as
 *               the labels of (left ∪ right), in that order, still needed
 *               outside the subtree or open in iy
 *   sliced    : n_sliced labels fixed per item (index slicing); each item of
 *               tb_solve_batch gives their 0/1 values
 * Replaces: uncompress (src/types.jl:75-79) + GenericTensorNetwork(...)
 * construction (src/dynamic_ob.jl:31).
 */
tb_status tb_plan_create(tb_ctx* ctx, int32_t n_labels, int32_t n_tensors, const int32_t* ix_off,
                         const int32_t* ix_lab, int32_t n_iy, const int32_t* iy, int32_t n_nodes,
                         const int32_t* children, const int32_t* node_iy_off,
                         const int32_t* node_iy_lab, int32_t n_sliced, const int32_t* sliced,
                         tb_plan** out);
void tb_plan_destroy(tb_plan* plan);
tb_status tb_plan_stats_get(const tb_plan* plan, tb_plan_stats* out);

/*
 * Output labels of internal node j (after slicing), for reading dumps.
 * Writes up to cap labels to labels_out and their count to *n_out.
 */
tb_status tb_plan_node_labels(const tb_plan* plan, int32_t node, int32_t cap, int32_t* labels_out,
                              int32_t* n_out);

/*
 * Bind vertex weights (n_labels floats, indexed by label) for the MIS leaf
 * tensors.  Replaces IndependentSet(g, weights) (src/dynamic_ob.jl:31).
 * Weights must be finite; in TB_DTYPE_I32 they must be integers.
 */
tb_status tb_plan_bind_mis(tb_plan* plan, const float* weights);

/*
 * tb_plan_bind_mis for n plans in one call: plan i takes the n_labels
 * weights at weights + offsets[i].  The weights only reach the device with
 * the next solve (one staged copy for the whole batch).
 */
tb_status tb_plan_bind_mis_batch(int32_t n, tb_plan* const* plans, const float* weights, const int64_t* offsets);

/*
 * Solve a batch of n items.  Item i contracts plans[i] with its sliced labels
 * fixed to slice_vals[sv_off_i .. sv_off_i + n_sliced_i) (items concatenated
 * in order; NULL when no plan slices), and returns
 *   out_item[i] = max(root tensor of item i) + r[i]
 * and *out_max = max_i out_item[i] (either pointer may be NULL; r may be NULL
 * for zeros).  A plan whose graph is empty (n_tensors == 0 is not allowed;
 * callers skip such items and use r directly, as contract_slices does at
 * src/dynamic_ob.jl:39-40).
 * Replaces: contract_slices (src/dynamic_ob.jl:36-48) and maximum(res)
 * (src/dynamic_ob.jl:27); with n == 1 and mode PLAIN, solve_slice.
 */
tb_status tb_solve_batch(tb_ctx* ctx, int32_t n, tb_plan* const* plans, const int8_t* slice_vals,
                         const float* r, float* out_item, float* out_max, int32_t mode);

/*
 * Score n_trees contraction trees of one network on the device: for tree t
 * (post-order pairs at children + t * 2 (n_tensors - 1)), out[4 t .. 4 t + 3]
 * = log2 time complexity (sum over nodes of 2^|labels(left) u labels(right)|),
 * space complexity (largest tensor rank), log2 read-write complexity and
 * log2 peak live elements of a post-order evaluation (every leaf live at the
 * start; each step allocates its output, then frees its operands).  Node
 * output labels follow the tb_plan_create rule.  Up to 4096 labels.
 * Replaces: contraction_complexity on candidate trees (src/types.jl:115-121,
 * sc_score src/branch.jl:132-147) and contraction_peak_memory
 * (src/utils.jl:197-219), evaluated one tree at a time on the host there.
 */
tb_status tb_score_trees(tb_ctx* ctx, int32_t n_labels, int32_t n_tensors, const int32_t* ix_off,
                         const int32_t* ix_lab, int32_t n_iy, const int32_t* iy, int32_t n_trees,
                         const int32_t* children, double* out);

/*
 * Choose the stream tile size (tile_bits 8..11) and the executor schedule
 * (persistent launch with 1..2 CTAs per SM and three run lengths, or
 * per-level launches with the stream kernel at 3 or 2 CTAs per SM, split-K
 * parts through partials or by atomic max) for this batch by running it with
 * each setting and
 * keeping the fastest; the chosen tiles stay in the plans and the schedule in
 * the context for TB_MODE_AUTO.  Arguments as tb_solve_batch.  Runs the batch
 * about 40 times.  No counterpart in the reference (its contraction has no
 * tunable schedule).
 */
tb_status tb_autotune(tb_ctx* ctx, int32_t n, tb_plan* const* plans, const int8_t* slice_vals,
                      const float* r, tb_tune_result* out);

/*
 * Contract one plan with explicit leaf tensors (host arrays, leaf i holding
 * 2^|ixs[i]| values, Tropical semantics: -inf is zero).  Writes the root
 * tensor (2^n_iy values, labels in iy order) to out.  The test form
 * `code(tensors...)` (test/utils.jl:34, test/decompose.jl:28).  Sliced plans
 * are not accepted here.
 */
tb_status tb_contract(tb_ctx* ctx, tb_plan* plan, const float* const* leaf_data, float* out,
                      int32_t mode);

/*
 * Run one item (MIS leaves) and copy every internal node's tensor to host:
 * node_out[j] receives 2^|labels(j)| values in the order tb_plan_node_labels
 * reports.  Entries of node_out may be NULL to skip a node.
 */
tb_status tb_dump_intermediates(tb_ctx* ctx, tb_plan* plan, const int8_t* slice_vals,
                                float* const* node_out, int32_t mode);

/*
 * Time the last tb_solve_batch's device work: kernel-only milliseconds of
 * the most recent call (CUDA events around the device work, excluding host
 * copies), and the number of kernel launches it made.
 */
tb_status tb_last_timing(const tb_ctx* ctx, double* device_ms, int64_t* launches);

/*
 * Standalone batched tropical GEMM (the K1 kernel), device pointers:
 *   C[m + M n + M N b] = max_k A[m + M k + M K b] + B[k + K n + K N b]
 * for b < batch; M, N, K powers of two >= 16.  `stream` is a cudaStream_t
 * (NULL: the default stream); the call only enqueues the kernel.
 * Uses the dtype of ctx.  Exposed for benchmarking the kernel at dense
 * square shapes.
 */
tb_status tb_gemm_device(tb_ctx* ctx, int64_t M, int64_t N, int64_t K, int64_t batch,
                         const void* A, const void* B, void* C, void* stream);

/*
 * Serving: continuous batching of MIS requests on one context.
 *
 * tb_serve_start starts a device-owner thread with a device pool of
 * pool_bytes (0: half the context budget) and at most max_items items in
 * flight (0: 4096).  tb_submit queues a request of n items (plans with their
 * slice values and r, as in tb_solve_batch) and returns at once; any thread
 * may submit, poll and wait.  The owner thread admits queued requests, whole
 * and in arrival order, as pool memory, item slots and one of four stream
 * slots free up; the requests admitted together form a cohort, which runs as
 * one batch of per-level launches on its slot's stream while the owner
 * thread goes on admitting, so requests that arrive while others run overlap
 * with them on the device; no step of it waits for the device.  A request
 * completes when the cohort holding its last item does.  A
 * request's result is the max over its items (as contract_slices + maximum,
 * src/dynamic_ob.jl:24-27).  Plans must outlive their requests and must not
 * be re-bound while a request uses them; while a server runs, call
 * tb_solve_batch on another context.  Has no single counterpart in the
 * reference (its requests are solved one at a time by dynamic_ob_mis).
 */
typedef struct tb_request tb_request;
tb_status tb_serve_start(tb_ctx* ctx, int64_t pool_bytes, int32_t max_items);
tb_status tb_serve_stop(tb_ctx* ctx);
tb_status tb_submit(tb_ctx* ctx, int32_t n, tb_plan* const* plans, const int8_t* slice_vals, const float* r,
                    tb_request** out);
tb_status tb_poll(tb_request* req, int32_t* done);
/* Wait up to timeout_ms (negative: no limit); result and submit-to-done
 * latency in milliseconds. */
tb_status tb_wait(tb_request* req, int32_t timeout_ms, float* out_max, double* latency_ms);
void tb_request_free(tb_request* req);
/* Cohorts launched (steps), kernel launches, requests completed and items in
 * flight. */
tb_status tb_serve_stats(tb_ctx* ctx, int64_t* steps, int64_t* launches, int64_t* completed, int64_t* active);

/*
 * tb_solve_static -- has no counterpart in the reference.
 *
 * One MIS contraction that allocates no device memory, for callers that
 * cannot call cudaMalloc (code running inside another runtime's memory pool
 * or allocator hooks, or handed only a stream).  All device memory it uses
 * lives in one fixed 64 MiB __device__ array that every GPU loading this
 * library holds until the process exits; networks whose arena does not fit
 * are refused with TB_ERR_UNSUPPORTED (tb_last_error(NULL) says why).
 * Arguments are those of tb_plan_create (no open or sliced labels, labels
 * derived) plus the vertex weights; the MIS value goes to *out_value (host).
 * Work is enqueued on `stream` (a cudaStream_t, NULL for the default stream)
 * with the plain per-contraction kernels, and the call returns after the
 * result is on the host.  The first call on a device looks up the array's
 * address; make it before any stream capture.  Calls share the array and
 * race if they overlap on the GPU: serialise them.
 */
tb_status tb_solve_static(int32_t n_labels, int32_t n_tensors, const int32_t* ix_off, const int32_t* ix_lab,
                          int32_t n_nodes, const int32_t* children, const float* weights, float* out_value,
                          void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TB_H */
