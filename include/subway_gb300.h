/*
 * subway_gb300.h — C ABI of the GB300-native out-of-HBM graph engine.
 *
 * This is the drop-in boundary for Subway's hot path: graph loading, the
 * per-iteration subgraph generation (activeness -> scan -> compaction ->
 * active-edge gather), partitioned host->device transfer under a device-memory
 * budget, and the BFS/SSSP/SSWP/CC/PR relaxation kernels in sync and async
 * variants.  Every entry point is plain C: pointers and sizes, no C++ or torch
 * types.  Every function returns an int status (SGW_OK = 0, negative = error)
 * and never exits the process; the reference calls exit() from inside library
 * code (shared/gpu_error_check.cuh:9-15, shared/graph.cu:171-175,
 * shared/partitioner.cu:66-70).
 *
 * Paths in the citations are relative to the Subway source tree.
 */
#ifndef SUBWAY_GB300_H
#define SUBWAY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SGW_OK          0
#define SGW_EINVAL     -1   /* bad argument                                  */
#define SGW_EIO        -2   /* file could not be opened / read / written     */
#define SGW_EFORMAT    -3   /* unsupported extension or malformed file       */
#define SGW_ENOMEM     -4   /* host allocation failed                        */
#define SGW_EBUDGET    -5   /* device budget too small for the vertex state  */
#define SGW_ECUDA      -6   /* a CUDA runtime call failed                    */
#define SGW_ETIMEOUT   -7   /* a bounded device-side wait gave up            */
#define SGW_ESTATE     -8   /* call made in the wrong engine state           */
#define SGW_ERANGE     -9   /* size beyond a documented limit                */

/* ---- algorithms and modes (subway/{bfs,sssp,sswp,cc,pr}-{sync,async}.cu) */
#define SGW_BFS   0
#define SGW_SSSP  1
#define SGW_SSWP  2
#define SGW_CC    3
#define SGW_PR    4
#define SGW_SYNC  0
#define SGW_ASYNC 1

/* DIST_INFINITY = UINT_MAX - 1 (shared/globals.hpp:27). */
#define SGW_DIST_INFINITY 4294967294u

typedef struct sgw_graph sgw_graph;
typedef struct sgw_engine sgw_engine;

/* Human-readable text for a status code, and the message of the last error
 * raised on the calling thread (empty string if none). */
const char *sgw_strerror(int status);
const char *sgw_last_error(void);

/* ---- graph (host side) --------------------------------------------------
 * The on-disk and in-memory edge records are the reference's:
 * OutEdge {u32 end} (4 B) and OutEdgeWeighted {u32 end; u32 w8} (8 B)
 * (shared/globals.hpp:33-40).  Binary CSR files are
 * [u32 n][u32 m][u32 nodePointer x n][edge x m]
 * (shared/graph.cu:39-52, tools/converter.cpp:88-95).  Graphs of 2^32 edges
 * or more, which that u32 header cannot describe, use .bcsr64 / .bwcsr64:
 * [u64 n][u64 m][u64 nodePointer x n][edge x m], the same records, every
 * field 8-byte aligned (no counterpart in the reference).  In memory a graph
 * keeps u32 node pointers below 2^32 edges and u64 ones from there on;
 * sgw_graph_node_pointer / sgw_graph_node_pointer64 return whichever it has
 * (the other is NULL).  Vertex ids stay u32 and out-degrees below 2^32.      */

/* Replaces Graph<E>::ReadGraph / GraphPR<E>::ReadGraph
 * (shared/graph.cu:32-197, :229-394).  The type is chosen by the extension:
 * .bcsr/.bcsr64/.el unweighted, .bwcsr/.bwcsr64/.wel weighted
 * (shared/graph.cu:37-53).
 * out-degree is derived for every vertex (the reference leaves
 * outDegree[n-2] unset, shared/graph.cu:179-181). */
int sgw_graph_load(const char *path, sgw_graph **out);

/* Maps a .bcsr/.bwcsr(64) file instead of reading it (shared/graph.cu:41-51
 * freads the whole file into pinned memory): the edge records stay in the
 * read-only file mapping, shared with the page cache, and only the n node
 * pointers are copied (plus the sentinel node_pointer[n] = m, which the file
 * does not hold).  The file is validated like sgw_graph_load (size, monotone
 * pointers, endpoints < n), which reads every record once.  The mapping is
 * released by sgw_graph_free.  Until then the file must not change: the
 * mapping is shared, so a process that truncates or rewrites it (the
 * converter writing to the same path, say) makes later reads fault (SIGBUS)
 * or see edges that were never validated; write a new file and rename it
 * over the old one instead, which leaves the mapped copy intact.
 * A .bwcsr file with an odd vertex count is read as by sgw_graph_load
 * instead, since its 8-byte records would not be 8-byte aligned. */
int sgw_graph_map(const char *path, sgw_graph **out);

/* Wraps a caller-owned host CSR without copying it.  node_pointer has n+1
 * entries (node_pointer[n] == m); edges holds m records of 4 B (weighted=0)
 * or 8 B (weighted=1).  The arrays must outlive the graph object and every
 * engine created on it.  Counterpart of the arrays that
 * Graph<E>::ReadGraph fills (shared/graph.cu:46-51). */
int sgw_graph_from_csr(uint32_t n, uint32_t m, const uint32_t *node_pointer,
                       const void *edges, int weighted, sgw_graph **out);
/* The same with u64 node pointers (any m; the arrays are borrowed as
 * above).  Engines on such a graph take the wide path whatever m is. */
int sgw_graph_from_csr64(uint32_t n, uint64_t m, const uint64_t *node_pointer,
                         const void *edges, int weighted, sgw_graph **out);

/* SGW_ERANGE for a graph of 2^32 edges or more: use sgw_graph_info64. */
int sgw_graph_info(const sgw_graph *g, uint32_t *n, uint32_t *m, int *weighted);
int sgw_graph_info64(const sgw_graph *g, uint32_t *n, uint64_t *m, int *weighted);
const uint32_t *sgw_graph_node_pointer(const sgw_graph *g);
const uint64_t *sgw_graph_node_pointer64(const sgw_graph *g);
const void *sgw_graph_edges(const sgw_graph *g);
/* outDegree[i] = nodePointer[i+1] - nodePointer[i] for all i
 * (shared/graph.cu:177-181 with every entry written). */
int sgw_graph_out_degree(const sgw_graph *g, uint32_t *out_degree);
/* Writes .bcsr/.bwcsr (tools/converter.cpp:88-95, :157-164), .bcsr64 /
 * .bwcsr64, or .el/.wel text, chosen by extension; SGW_ERANGE for a u32
 * file of a graph with 2^32 edges or more. */
int sgw_graph_save(const sgw_graph *g, const char *path);
/* Removes vertex v's out-edges (the rows after it move down, m shrinks; the
 * node pointers keep their width).  Only for a graph whose arrays the library
 * owns (sgw_graph_load, the generators), and not while an engine or batch
 * uses it.  The apps' --subway-compat uses it on vertex n - 2, whose
 * out-degree the reference never writes (shared/graph.cu:179-181), so that
 * its edges are ignored there. */
int sgw_graph_clear_out_edges(sgw_graph *g, uint32_t v);
void sgw_graph_free(sgw_graph *g);

/* ---- engine --------------------------------------------------------------- */
#define SGW_OPT_PROFILE   0x1u  /* time every kernel class with CUDA events   */
#define SGW_OPT_NO_OVERLAP 0x2u /* one edge buffer, no copy/compute overlap   */
/* Weighted graphs are moved as one 32-bit word per edge, (w8 << b) | end with
 * b = bits of the largest vertex id, whenever every weight fits in 32 - b
 * bits (a packed copy of the edges is built in host memory at engine
 * creation).  This flag keeps the reference's 8-byte records instead. */
#define SGW_OPT_NO_PACK    0x4u
/* Gather host records one per thread instead of as aligned 16-byte words. */
#define SGW_OPT_SCALAR_GATHER 0x8u
/* Expand frontier edges in CTA tiles of 256 sources (k_relax_tile) instead
 * of warp tiles of 32 (k_relax_warp). */
#define SGW_OPT_CTA_TILES 0x10u
/* Weighted graphs whose weights do not pack beside the vertex id, but are
 * all below 256, move as a u32 destination stream plus a u8 weight stream
 * (5 bytes per edge; BFS/CC/PR move only the destinations).  This flag uses
 * that split form even where the packed word would fit. */
#define SGW_OPT_SPLIT_WEIGHTS 0x20u
/* sgw_batch_create: a batch runs either as one cooperative launch whose
 * blocks loop over the iterations behind grid barriers (the persistent form;
 * a barrier waits at most 2 s, after which the run returns SGW_ETIMEOUT), or
 * as a CUDA graph whose conditional WHILE node repeats one iteration's
 * kernels.  By default SSSP batches take the persistent form and BFS batches
 * the graph (measured best); these flags force one form for both. */
#define SGW_OPT_BATCH_PERSISTENT 0x40u
#define SGW_OPT_BATCH_GRAPH 0x80u
/* The engine's host transfer copy in ordinary pageable pages instead of
 * pinned cudaHostAlloc memory, on devices that read pageable memory through
 * the host page tables (GB300 with its Grace host; elsewhere the flag is
 * ignored): the filling threads' first touch replaces the driver's page
 * pinning, so engine creation and destruction take about half as long (RMAT-28:
 * 0.47-0.58 s against 1.0-1.08 s to create, 0.08 against 0.16 s to destroy),
 * while a run is as fast under the plain schedule and 4-7% slower under the
 * learned one.  Whole-range and hub copies then run as a copy kernel instead
 * of DMA.  The drop-in apps, which answer one query per process, set it. */
#define SGW_OPT_PAGEABLE_COPY 0x100u
/* No transfer copy at all where the device reads pageable memory through the
 * host page tables and the graph's records are the library's own (from
 * sgw_graph_load of any format, or the generators; not a file mapping or a
 * caller's arrays): the gather and copy kernels read the records in place,
 * at their full size (4 or 8 bytes per edge, not packed or split).  Engine
 * creation then touches no edge; each run moves up to 8/5 as many bytes as
 * from the split copy.  Otherwise the flag is ignored (a transfer copy is
 * made, pageable with SGW_OPT_PAGEABLE_COPY).  The drop-in apps set both. */
#define SGW_OPT_GRAPH_IN_PLACE 0x200u
/* sched_flags: the learned policy's inner cap also covers compacted ranges */
#define SGW_SCHED_CAP_COMPACT 0x1u
/* sched_flags: transfer active vertices that cannot push, as the reference's
 * schedule does (for measuring what skipping them saves) */
#define SGW_SCHED_KEEP_IDLE 0x2u

typedef struct sgw_engine_opts {
  /* Device-memory budget in bytes for everything the engine allocates.
   * 0 = the reference's rule: 0.9 * (totalGlobalMem - 32 n) bytes of edges
   * (shared/subgraph.cu:24-28) plus the vertex state. */
  uint64_t budget_bytes;
  int32_t device;          /* CUDA device ordinal (--device)                  */
  uint32_t flags;          /* SGW_OPT_*                                       */
  uint32_t inner_batch;    /* async inner iterations launched per host check  */
  uint32_t tile_degree_max;/* sources above this degree go to the chunk list  */
  uint32_t chunk_edges;    /* edges per chunk-list item (multiple of 32)      */
  uint32_t gather_ctas;    /* CTAs of the gather kernel, 0 = 2 per SM (3 per SM
                              under the learned policy)                      */
  uint32_t num_buffers;    /* device edge buffers sharing the budget, 0 = 2
                              (1 with SGW_OPT_NO_OVERLAP), at most 8          */
  /* Learned policy, async mode: a range whose predicted active-edge fraction
   * for the next global iteration is at least sched_active_permille / 1000
   * (0 = 1) runs at most sched_inner inner iterations (0 = 3) now, since what
   * further passes would settle is likely to be redone when it is relaxed
   * again; other ranges run to local convergence.  Without
   * SGW_SCHED_CAP_COMPACT the cap only covers ranges that stay in their edge
   * buffer (their leftover sources cost no transfer).
   * sched_active_permille > 1000 turns the cap off.  Defaults: 3, 1,
   * SGW_SCHED_CAP_COMPACT. */
  uint32_t sched_inner;
  uint32_t sched_active_permille;
  uint32_t sched_flags;    /* SGW_SCHED_*                                     */
  /* Learned policy: each global iteration takes the active vertices with the
   * lowest values (highest for SSWP) up to about sched_defer_permille / 1000
   * of the graph's edges and leaves the rest active for later iterations.
   * 0 = automatic: 250 when the graph's edge records exceed four times the
   * edge-buffer space, else the whole frontier; above 1000 = always the
   * whole frontier.  Under this policy active vertices that cannot push
   * (value INF for BFS/SSSP, 0 for SSWP) are never transferred. */
  uint32_t sched_defer_permille;
  /* The host transfer copy is allocated in pinned chunks of
   * 2^transfer_chunk_log2 bytes (0 = 30, i.e. 1 GiB; at most 64 chunks per
   * stream, larger chunks if needed), two chunks at a time. */
  uint32_t transfer_chunk_log2;
  /* Most edges one generate queues: the active vertices of whole 4096-vertex
   * tiles, in vertex order, up to this many edges (the first tile with edges
   * always); the rest stay active for the next iteration, which the
   * BFS/SSSP/SSWP/CC answers do not depend on (PageRank keeps their
   * residuals for the next round).  0 = 2^31 for graphs of 2^32 edges or
   * more (queue positions are u32), else no limit. */
  uint32_t generate_edge_limit;
} sgw_engine_opts;

void sgw_engine_opts_default(sgw_engine_opts *opts);

/* Creates the device vertex state and edge buffers under the budget and
 * registers the graph's host edges for device access.  Replaces the
 * allocation side of Graph<E>::ReadGraph (shared/graph.cu:187-190),
 * Subgraph<E>::Subgraph (shared/subgraph.cu:9-42) and
 * SubgraphGenerator<E>::SubgraphGenerator (shared/subgraph_generator.cu:100-126). */
int sgw_engine_create(const sgw_graph *g, const sgw_engine_opts *opts,
                      sgw_engine **out);
int sgw_engine_destroy(sgw_engine *e);

/* max_partition_size: edges one device edge buffer holds
 * (Subgraph<E>::max_partition_size, shared/subgraph.cu:24-28). */
int sgw_engine_max_partition_size(const sgw_engine *e, uint64_t *edges);
/* Device bytes the engine holds (always <= the budget). */
int sgw_engine_device_bytes(const sgw_engine *e, uint64_t *bytes);
/* Bytes of the engine's host transfer copy (0 when it reads the graph's
 * records in place, SGW_OPT_GRAPH_IN_PLACE). */
int sgw_engine_host_copy_bytes(const sgw_engine *e, uint64_t *bytes);

typedef struct sgw_run_params {
  int32_t algo;            /* SGW_BFS .. SGW_PR                               */
  int32_t mode;            /* SGW_SYNC / SGW_ASYNC                            */
  uint32_t source;         /* --source (ignored by CC and PR)                 */
  float pr_init;           /* initial delta, 0.15 (subway/pr-sync.cu:33)      */
  float pr_acc;            /* activation threshold, 0.01 (subway/pr-sync.cu:34) */
  float pr_damping;        /* 0.85 (shared/gpu_kernels.cu:239)                */
  uint32_t max_inner;      /* async: inner iterations per partition visit,
                              0 = until the partition converges (reference)  */
  uint32_t reserved[7];
} sgw_run_params;

void sgw_run_params_default(sgw_run_params *p, int algo, int mode, uint32_t source);

typedef struct sgw_run_stats {
  uint32_t global_iterations;   /* "Number of iterations" (subway/bfs-sync.cu:94) */
  uint32_t partitions;          /* partitions processed, summed over iterations */
  uint64_t inner_iterations;    /* async inner iterations, summed               */
  uint64_t active_vertices;     /* queued (degree > 0) vertices, summed         */
  uint64_t active_edges;        /* edges of queued vertices, summed             */
  uint64_t h2d_bytes;           /* bytes read from host memory by the device    */
  uint64_t d2h_bytes;           /* bytes copied device -> host                  */
  uint64_t reached_edges;       /* edges whose source has a final label that is
                                   not the initial one (Graph500 m_reached)     */
  double ms_device;             /* CUDA-event time of the processing loop       */
  double ms_generate;           /* SGW_OPT_PROFILE: per kernel class totals     */
  double ms_partition;
  double ms_gather;             /* the gather kernel (k_gather_v) alone         */
  double ms_relax;
  uint64_t launches;            /* kernels launched by the run                  */
  uint64_t gather_launches;
  uint64_t relax_launches;
  uint64_t generate_launches;
  uint64_t relaxed_edges;       /* edges expanded by the relaxation kernels     */
  uint64_t relaxed_sources;     /* sources whose edges were expanded            */
  uint64_t gather_bytes;        /* host bytes the gather kernel read (the same
                                   count is written to HBM); h2d_bytes minus
                                   this is what DMA copies moved                */
  double ms_stream;             /* SGW_OPT_PROFILE: DMA copies of whole ranges
                                   and of split-vertex pieces                   */
} sgw_run_stats;

/* One whole application run: the init loops, the first generate, the
 * global-iteration / partition / inner-iteration loops and the final value
 * read-back of subway/<algo>-<mode>.cu (e.g. subway/sssp-async.cu:38-127).
 * out_values: host buffer of n uint32 (float for PR).  stats may be NULL. */
int sgw_run(sgw_engine *e, const sgw_run_params *p, void *out_values,
            sgw_run_stats *stats);

/* ---- step API: the reference's role classes, one call per role ------- */

/* The per-app initial state (values, label1/label2; PR delta/value), e.g.
 * subway/sssp-async.cu:38-51 and :59-64, and the first generate
 * (:57).  Leaves the engine ready for sgw_partition. */
int sgw_state_init(sgw_engine *e, const sgw_run_params *p);
/* SubgraphGenerator<E>::generate (shared/subgraph_generator.cu:128-204,
 * :209-285): activeness, scan, compaction.  Returns the number of queued
 * vertices and their edges. */
int sgw_generate(sgw_engine *e, uint32_t *num_active_nodes,
                 uint64_t *num_active_edges);
/* Partitioner<E>::partition (shared/partitioner.cu:12-91). */
int sgw_partition(sgw_engine *e, uint32_t *num_partitions);
int sgw_partition_info(const sgw_engine *e, uint32_t i, uint32_t *from_node,
                       uint32_t *from_edge, uint32_t *node_size,
                       uint64_t *edge_size);
/* One partition of one global iteration: the transfer, the label hand-off
 * (moveUpLabels / mixLabels, shared/gpu_kernels.cu:515-534) and the
 * relaxation kernel or async inner loop (subway/sssp-async.cu:85-117). */
int sgw_process_partition(sgw_engine *e, uint32_t i, uint32_t *inner_iterations);
/* Device -> host copy of the values (subway/sssp-async.cu:127). */
int sgw_read_values(sgw_engine *e, void *out_values);
/* PR only: the engine's double-precision values. */
int sgw_read_values_f64(sgw_engine *e, double *out_values);
/* The compacted active queue of the last generate: activeNodes and
 * activeNodesPointer (shared/subgraph.cuh:19-20); ptr has count+1 entries. */
int sgw_read_active(sgw_engine *e, uint32_t *nodes, uint32_t *ptr,
                    uint32_t capacity, uint32_t *count);

/* Statistics accumulated since the last sgw_state_init / sgw_run. */
int sgw_get_stats(const sgw_engine *e, sgw_run_stats *stats);

/* ---- per-partition trace ----------------------------------------------
 * One record per processed partition.  The reference prints the inner
 * iteration count of each async partition (subway/sssp-async.cu:117); the
 * trace carries that and the transfer volume, and is the training data of
 * the learned scheduler. */
typedef struct sgw_trace_rec {
  uint32_t global_iteration;      /* 1-based                                  */
  uint32_t partition;             /* index within the global iteration        */
  uint32_t num_partitions;        /* partitions in this global iteration      */
  uint32_t inner_iterations;      /* relaxation passes run on the partition   */
  uint32_t active_nodes;          /* queued vertices of the partition         */
  uint32_t first_vertex;          /* lowest vertex id of the partition        */
  uint64_t active_edges;          /* edges of those vertices                  */
  uint64_t iteration_active_nodes;/* queued vertices of the whole iteration   */
  uint64_t iteration_active_edges;
  uint64_t bytes_h2d;             /* bytes read from host for the partition   */
  uint32_t transfer;              /* 0 compacted gather, 1 range stream, 2 split vertex */
  uint32_t reserved;
} sgw_trace_rec;

/* Records are kept from the next sgw_state_init / sgw_run on while enabled. */
int sgw_trace_enable(sgw_engine *e, int on);
int sgw_trace_count(const sgw_engine *e, uint64_t *count);
int sgw_trace_read(const sgw_engine *e, sgw_trace_rec *out, uint64_t capacity,
                   uint64_t *count);
/* The trace as a CSV file (a header line, then one line per record, the
 * fields in struct order; `reserved` left out).  sgw_trace_save writes the
 * engine's records; sgw_trace_write_csv any array of them. */
int sgw_trace_save(const sgw_engine *e, const char *path);
int sgw_trace_write_csv(const sgw_trace_rec *recs, uint64_t count, const char *path);

/* Partition planning on the host: the greedy split of a compacted active
 * queue (prefix array ptr of count+1 entries) into runs whose edge count is
 * at most cap; a vertex with more than cap edges gets a run of its own.
 * Same routine the device planner runs.  Replaces the binary search of
 * shared/partitioner.cu:29-91 (which never ends when one vertex exceeds the
 * budget).  Returns the number of runs; from/size arrays get one entry each
 * (capacity entries at most). */
int sgw_plan_partitions(const uint32_t *ptr, uint32_t count, uint64_t cap,
                        uint32_t *from_node, uint32_t *node_size,
                        uint32_t capacity, uint32_t *num_partitions);

/* Number of CUDA devices visible (0 on a machine without a GPU). */
int sgw_device_count(int *count);
/* Streaming multiprocessors and global memory bytes of a device. */
int sgw_device_info(int device, uint32_t *sm_count, uint64_t *total_bytes);

/* ---- learned scheduler ------------------------------------------------------
 * No counterpart in the reference, whose only schedule is: compact every
 * active vertex's edges, cut the queue greedily into budget-sized partitions,
 * process them in vertex order, iterate each async partition to convergence
 * (SGW_POLICY_PLAIN, the default, which this engine reproduces).
 *
 * SGW_POLICY_LEARNED cuts the vertex ids into static ranges that each fit one
 * edge buffer.  After every generate step a kernel counts each range's active
 * vertices and edges and evaluates the network below on five features
 * (active vertex fraction, active edge fraction, growth of the active edges
 * since the previous iteration, iteration index, range edge count), giving
 * the predicted active edge fraction of the range in the next iteration.
 * The host then, per active range: processes it from HBM if a buffer still
 * holds it (no transfer); else streams the whole range (one DMA copy, and the
 * buffer keeps it) when the extra bytes now are covered by the predicted
 * bytes saved next iteration, or gathers only its active edges; evicts the
 * buffer with the lowest predicted saving; and orders resident ranges first.
 * Results are identical to the plain policy (the schedule changes, the
 * fixpoint does not).  With model == NULL the prediction is the current
 * active edge fraction.
 *
 * The network: 5 -> 64 -> 64 -> 1, ReLU, sigmoid output, BF16 weights, FP32
 * accumulation, trained by binary cross-entropy with Adam on FP32 masters,
 * all in hand-written kernels.  Parameters are flat FP32 arrays in the order
 * W1[64][5], b1[64], W2[64][64], b2[64], W3[64], b3. */
typedef struct sgw_mlp sgw_mlp;
#define SGW_MLP_INPUTS 5
#define SGW_MLP_HIDDEN 64
#define SGW_MLP_PARAMS 4609
#define SGW_POLICY_PLAIN 0
#define SGW_POLICY_LEARNED 1

int sgw_mlp_create(int device, uint64_t seed, sgw_mlp **out);
int sgw_mlp_destroy(sgw_mlp *m);
/* Sets the FP32 masters (and their BF16 copy) and resets the optimiser. */
int sgw_mlp_set_params(sgw_mlp *m, const float *params);
/* The BF16 weights the passes use, widened to FP32. */
int sgw_mlp_get_params(const sgw_mlp *m, float *params);
/* Host arrays: x is n x SGW_MLP_INPUTS, y and t have n entries. */
int sgw_mlp_forward(sgw_mlp *m, const float *x, uint32_t n, float *y);
int sgw_mlp_gradient(sgw_mlp *m, const float *x, const float *t, uint32_t n,
                     float *grad, float *loss);
int sgw_mlp_train(sgw_mlp *m, const float *x, const float *t, uint32_t n,
                  uint32_t steps, float lr, float *loss);
int sgw_mlp_save(const sgw_mlp *m, const char *path);
int sgw_mlp_load(int device, const char *path, sgw_mlp **out);

/* Takes effect from the next run; the model's weights are copied into the
 * engine's device budget, so the model may be destroyed afterwards. */
int sgw_set_policy(sgw_engine *e, int policy, const sgw_mlp *model);
/* Edge buffers the learned policy should be created with for this graph and
 * budget: 3 when a third of the edge space still holds at least 15% of the
 * graph's edges (one range can then stay resident while two buffers keep
 * transfers and relaxation overlapped), else 2 (larger partitions pay more
 * than residency of a small slice). */
int sgw_sched_buffers(const sgw_graph *g, uint64_t budget_bytes, uint32_t *num_buffers);
/* Host-to-device DMA rate (GB/s) from the engine's transfer copy, timed at
 * engine creation (-1 when the copy is too small to time).  The learned
 * policy streams whole ranges only when it is at least 120 GB/s. */
int sgw_engine_dma_rate(const sgw_engine *e, double *gbs);

/* Per range and global iteration of a SGW_POLICY_LEARNED run (recorded while
 * the trace is enabled): the features, the prediction and what was done. */
#define SGW_ACT_SKIP 0      /* no active vertex                               */
#define SGW_ACT_RESIDENT 1  /* processed from a buffer that still held it     */
#define SGW_ACT_STREAM 2    /* whole range copied, kept resident              */
#define SGW_ACT_COMPACT 3   /* active edges gathered                          */
#define SGW_ACT_SPLIT 4     /* one vertex larger than a buffer, in pieces     */
typedef struct sgw_range_rec {
  uint32_t global_iteration;
  uint32_t range;
  uint32_t active_nodes;
  uint32_t range_nodes;
  uint32_t active_edges;
  uint32_t range_edges;
  uint32_t action;
  uint32_t inner_iterations;
  float features[5];
  float predicted;
  uint64_t bytes_h2d;
} sgw_range_rec;
int sgw_range_trace_count(const sgw_engine *e, uint64_t *count);
int sgw_range_trace_read(const sgw_engine *e, sgw_range_rec *out, uint64_t capacity,
                         uint64_t *count);

/* ---- batched multi-source queries ------------------------------------------
 * No counterpart in the reference, which runs one source per process
 * (subway/bfs-sync.cu, subway/sssp-sync.cu).  Up to 64 BFS or SSSP queries
 * share one traversal of a graph held in HBM: per vertex one distance per
 * query lane and a 64-bit lane mask for the current and next frontier.  A
 * batch is one CUDA-graph launch whose conditional WHILE node repeats the
 * frontier/relax iteration on the device until no lane improves.  Results
 * are bit-exact with single-source runs.
 * opts: budget_bytes (admission: SGW_EBUDGET if the graph, lanes x n
 * distances and the work lists do not fit), device, chunk_edges (edges per
 * work item, default 256), flags (SGW_OPT_NO_PACK). */
typedef struct sgw_batch sgw_batch;
typedef struct sgw_batch_stats {
  uint32_t iterations;      /* frontier iterations of the batch               */
  uint32_t queries;
  double ms_device;         /* CUDA-event time of the traversal               */
  double ms_wall;           /* the whole call, results copied to the host     */
  uint64_t d2h_bytes;
  uint64_t reserved[4];
} sgw_batch_stats;

/* lanes: 32 or 64 (the widest batch). */
int sgw_batch_create(const sgw_graph *g, const sgw_engine_opts *opts, uint32_t lanes,
                     sgw_batch **out);
int sgw_batch_destroy(sgw_batch *b);
int sgw_batch_device_bytes(const sgw_batch *b, uint64_t *bytes);
/* algo: SGW_BFS or SGW_SSSP.  out: host array of nsrc x n uint32, query i's
 * distances at out[i * n .. i * n + n); NULL leaves them in the batch's own
 * pinned buffer (faster: no pageable copy), see sgw_batch_results. */
int sgw_batch_run(sgw_batch *b, int algo, const uint32_t *sources, uint32_t nsrc,
                  uint32_t *out, sgw_batch_stats *stats);
/* sgw_batch_run with 16-bit answers (no reference counterpart): distances or
 * levels as uint16, unreached = 0xffff, half the bytes copied to the host
 * (the copy-out bounds a server on large graphs).  out: nsrc x n uint16,
 * or NULL to leave them in the batch's pinned buffer (sgw_batch_results,
 * read as uint16).  A reached value of 0xffff or more returns SGW_ERANGE
 * (the answers are then not usable; run sgw_batch_run). */
int sgw_batch_run_u16(sgw_batch *b, int algo, const uint32_t *sources, uint32_t nsrc,
                      uint16_t *out, sgw_batch_stats *stats);
/* Failure-path check of the persistent form (no reference counterpart): runs
 * its kernel once with grid barriers that wait for one block more than the
 * launch has, so every wait runs out after wait_ns (1 ns .. 1 s).  Returns
 * SGW_ETIMEOUT when the kernel gave up and the device stayed usable; the
 * batch object can be used again afterwards. */
int sgw_batch_check_wait_timeout(sgw_batch *b, uint64_t wait_ns);
/* The batch's pinned result buffer (lanes x n, lane-major), valid until the
 * next sgw_batch_run or sgw_batch_destroy. */
int sgw_batch_results(const sgw_batch *b, const uint32_t **results);

/* ---- allocation-free compaction ------------------------------------------
 * No counterpart in the reference (its generate step allocates its scan
 * buffers through thrust, shared/subgraph_generator.cu:138-150).
 *
 * For callers that cannot call cudaMalloc: a host framework that already owns
 * every byte of device memory through its own pool.  It runs the engine's activeness -> scan -> compaction kernel on
 * device arrays the caller provides (label1, label2 bytes of n vertices;
 * node_pointer of n+1 entries; queue of n and ptr of n+1 entries), with the
 * scan's tile state in a static device array inside this library
 * (about 321 KB, held by every GPU that loads the library until exit).  It
 * calls no allocating routine.
 *  - n must be at most SGW_NOALLOC_MAX_VERTICES; larger n returns SGW_ERANGE.
 *  - consume != 0 clears the labels of queued vertices (the sync form);
 *    labels of active vertices with no out-edges are always cleared.
 *  - The first call on a device looks up the static array's device address
 *    (cudaGetSymbolAddress) with that device current.
 *  - Every call shares the one static array: calls whose work overlaps on
 *    the GPU (other streams, other host threads) race; serialise them.
 *  - stream is a cudaStream_t (NULL = legacy default stream); every call
 *    synchronises it to return the counts on the host, so it cannot be
 *    recorded into a stream capture or a CUDA graph. */
#define SGW_NOALLOC_MAX_VERTICES 67108864u
int sgw_generate_noalloc(uint8_t *d_label1, uint8_t *d_label2,
                         const uint32_t *d_node_pointer, uint32_t n, int consume,
                         uint32_t *d_queue, uint32_t *d_ptr, void *stream,
                         uint32_t *num_active, uint64_t *num_active_edges);

/* Host-link copy bandwidth of `device` in GB/s: pinned host -> device and
 * device -> host cudaMemcpyAsync of `bytes`, best of `iters` (the
 * denominator of the gather kernel's roofline). */
int sgw_probe_link(int device, uint64_t bytes, int iters, double *h2d_gbs,
                   double *d2h_gbs);

#ifdef __cplusplus
}
#endif
#endif /* SUBWAY_GB300_H */
