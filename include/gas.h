/*
 * gas.h -- C ABI of libgas, the GB300 (sm_103a) Gather-Apply-Scatter engine.
 *
 * Plain C: pointers, sizes and status codes only.  Every entry point returns a
 * gas_status_t; gas_last_error() gives a one-line description of the last
 * failure on the calling thread.  Each declaration names the reference
 * interface it replaces (paths inside dipanjans12/GraphReduce).
 *
 * Three layers:
 *   1. host edge lists: graph I/O (.gr), synthetic R-MAT / Erdos-Renyi /
 *      grid-island generators, source pickers, CSR construction;
 *   2. the engine (GASEngineGPU's step API) for the reference's four vertex
 *      programs built in (BFS, SSSP, CC, PageRank) and for user programs
 *      compiled through include/gpugas.h;
 *   3. whole-algorithm runs on a device-resident graph (the fast schedules,
 *      device-side convergence, CUDA-graph iteration loop).
 *
 * Threading: an engine or graph handle is used by one host thread at a time.
 * Streams: every call that launches work takes a cudaStream_t passed as
 * void* (NULL = the legacy default stream, which is what the reference's
 * apps rely on, bfs.cu:83-90).  Calls that return host values synchronise
 * that stream.
 */
#ifndef GAS_H_
#define GAS_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GAS_OK = 0,
  GAS_ERR_INVALID = 1,     /* bad argument (null pointer, id out of range...) */
  GAS_ERR_NOMEM = 2,       /* host or device allocation failed */
  GAS_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  GAS_ERR_ITER_CAP = 4,    /* iteration cap reached before convergence */
  GAS_ERR_IO = 5,          /* file could not be read / written / parsed */
  GAS_ERR_STATE = 6,       /* call out of order (e.g. run before setGraph) */
  GAS_ERR_UNSUPPORTED = 7, /* operation not available for this program */
  GAS_ERR_DEVICE = 8,      /* a kernel reported an error through its flag */
  GAS_ERR_TOO_LARGE = 9    /* sizes beyond the 32-bit index space */
} gas_status_t;

/* Human-readable name of a status code. */
const char *gas_status_string(gas_status_t s);
/* Detail of the last failure on this thread ("" if none). */
const char *gas_last_error(void);
/* Library version string. */
const char *gas_version(void);

/* ======================================================================= */
/* 1. Host edge lists (graphio.h / graphio.cpp, util.cuh)                  */
/* ======================================================================= */

/* An edge list in host memory: nV vertices, nE directed edges, optional
 * 32-bit edge data (weights).  Generators return edges sorted by (src,dst). */
typedef struct gas_edge_list gas_edge_list;

/* Wrap copies of caller arrays (weights may be NULL).
 * Replaces the std::vector<int> srcs/dsts/edgeValues triple that
 * loadGraph fills (graphio.h:63-67). */
gas_status_t gas_edge_list_create(int32_t nV, int64_t nE, const int32_t *srcs,
                                  const int32_t *dsts, const int32_t *weights,
                                  gas_edge_list **out);
void gas_edge_list_destroy(gas_edge_list *el);
int32_t gas_edge_list_num_vertices(const gas_edge_list *el);
int64_t gas_edge_list_num_edges(const gas_edge_list *el);
const int32_t *gas_edge_list_srcs(const gas_edge_list *el);
const int32_t *gas_edge_list_dsts(const gas_edge_list *el);
const int32_t *gas_edge_list_weights(const gas_edge_list *el); /* NULL if none */

/* Seeded R-MAT graph: 2^scale vertices, edge_factor * 2^scale samples with
 * quadrant probabilities (a, b, c, 1-a-b-c), no vertex permutation.  Self
 * loops and duplicates are removed; symmetrize adds the reverse of every
 * edge first.  No reference counterpart (the reference reads files only). */
gas_status_t gas_rmat(int32_t scale, int32_t edge_factor, double a, double b,
                      double c, uint64_t seed, int32_t symmetrize,
                      gas_edge_list **out);

/* Seeded Erdos-Renyi graph with n_samples uniform (src, dst) draws, self
 * loops and duplicates removed.  No reference counterpart. */
gas_status_t gas_erdos_renyi(int32_t nV, int64_t n_samples, uint64_t seed,
                             int32_t symmetrize, gas_edge_list **out);

/* Append n_islands disjoint side x side 4-neighbour grids (both directions)
 * after the existing vertices, the way createCCGraph.cpp:36-44 concatenates
 * graphs at vertex offsets. */
gas_status_t gas_edge_list_append_grid_islands(gas_edge_list *el,
                                               int32_t n_islands,
                                               int32_t side);

/* Give every edge a weight uniform in [lo, hi], drawn from (seed, min(u,v),
 * max(u,v)) so both directions of an undirected edge agree. */
gas_status_t gas_edge_list_set_uniform_weights(gas_edge_list *el, int32_t lo,
                                               int32_t hi, uint64_t seed);

/* The first vertex of maximum out-degree (bfs.cu:175-195, sssp.cu:148-168). */
gas_status_t gas_edge_list_max_out_degree_vertex(const gas_edge_list *el,
                                                 int32_t *vertex,
                                                 int32_t *degree);

/* k distinct vertices drawn uniformly (seeded) from the largest weakly
 * connected component.  No reference counterpart. */
gas_status_t gas_edge_list_sample_sources(const gas_edge_list *el, int32_t k,
                                          uint64_t seed, int32_t *out);

/* Lonestar binary CSR ".gr" files (graphio.cpp:265-272 format).
 * gas_gr_write replaces writeGraph_binaryCSR (graphio.cpp:365-413) and always
 * writes 4-byte edge data (zeros when the list has none) because the
 * reference reader rejects files without it (graphio.cpp:298-307).
 * gas_gr_read replaces loadGraph_binaryCSR with expand=true
 * (graphio.cpp:274-362); files with 0-byte edge data are accepted too. */
gas_status_t gas_gr_write(const char *path, const gas_edge_list *el);
gas_status_t gas_gr_read(const char *path, gas_edge_list **out);

/* Text formats of graphio.cpp (plain files; gzip is not read):
 * gas_mtx_read replaces loadGraph_MatrixMarket (graphio.cpp:190-270):
 * "%%MatrixMarket matrix coordinate <type> <symmetry>" header, '%' comments,
 * the size line ignored, 1-based ids, self loops dropped, "symmetric" /
 * "skew-symmetric" (and value-less "hermitian") add the reverse edge right
 * after each edge (skew: negated value), values parsed as float and
 * truncated to int, "pattern" gives no edge data, "complex" is rejected,
 * nV = largest id + 1 (a self loop of a valued file does not count, as in
 * loadGraph_common, graphio.cpp:69-176).  gas_snap_read replaces
 * loadGraph_GraphLabSnap (graphio.cpp:178-188): '#' comments, 0-based
 * "src dst" lines, self loops dropped, no edge data.  gas_mtx_write replaces
 * writeGraph_mtx (graphio.cpp:416-437).  gas_graph_read dispatches on the
 * extension like loadGraph (graphio.cpp:441-473): .edge, .mtx, .gr. */
gas_status_t gas_mtx_read(const char *path, gas_edge_list **out);
gas_status_t gas_snap_read(const char *path, gas_edge_list **out);
gas_status_t gas_mtx_write(const char *path, const gas_edge_list *el);
gas_status_t gas_graph_read(const char *path, gas_edge_list **out);

/* edgeListToCSR (util.cuh:80-111): offsets[nV+1], out[nE] = vals in key
 * order, perm[nE] = original edge index (out / perm may be NULL).  Edges of
 * one key keep their edge-list order (stable). */
gas_status_t gas_edge_list_to_csr(int32_t nV, int64_t nE, const int32_t *keys,
                                  const int32_t *vals, int32_t *offsets,
                                  int32_t *out, int32_t *perm);

/* ======================================================================= */
/* 2. Engine: GASEngineGPU (gpugas.h:1025-1809) as a C handle              */
/* ======================================================================= */

typedef enum {
  GAS_PROG_USER = 0,     /* user Program compiled through include/gpugas.h */
  GAS_PROG_BFS = 1,      /* bfs.cu:31-80            VertexData int32 depth  */
  GAS_PROG_SSSP = 2,     /* sssp.cu:25-66           int32 dist, int32 weight */
  GAS_PROG_CC = 3,       /* connected_component.cu:25-63  int32 label       */
  GAS_PROG_PAGERANK = 4  /* pagerank.cu:27-73  {float rank; int32 numOutEdges} */
} gas_program_t;

typedef struct gas_engine gas_engine;

/* GASEngineGPU() (gpugas.h:1129-1163) for a built-in program. */
gas_status_t gas_engine_create(gas_program_t program, gas_engine **out);

/* GASEngineGPU<Program>() for a user program: sizes of VertexData,
 * GatherResult and EdgeData (EdgeData may be an empty struct: pass its
 * sizeof).  Gather/apply kernels are then launched by include/gpugas.h. */
gas_status_t gas_engine_create_user(size_t vertex_bytes, size_t gather_bytes,
                                    size_t edge_bytes, gas_engine **out);

/* ~GASEngineGPU() (gpugas.h:1165-1193). */
void gas_engine_destroy(gas_engine *e);

/* setGraph (gpugas.h:1314-1503): copies vertex data (nV records) and edge
 * data (nE records, may be NULL) to the device and builds CSC (gather) and
 * CSR (scatter) there from the edge list.  The host vertex array stays
 * registered as the destination of gas_engine_get_results.  May be called
 * again on the same engine (sssp.cu:85).  The built-in SSSP needs int32
 * weights in [0, 100000] (its gatherZero INT_MAX - 100000 leaves that
 * margin, sssp.cu:32-33); others return GAS_ERR_INVALID. */
gas_status_t gas_engine_set_graph(gas_engine *e, int32_t nV, void *vertex_data,
                                  int64_t nE, const void *edge_data,
                                  const int32_t *srcs, const int32_t *dsts,
                                  void *stream);

/* setActive(start, end) (gpugas.h:1524-1546): active = [start, end). */
gas_status_t gas_engine_set_active(gas_engine *e, int32_t start, int32_t end,
                                   void *stream);

/* countActive() (gpugas.h:1548-1551): size of the active set (host value). */
gas_status_t gas_engine_count_active(gas_engine *e, int32_t *n_active);

/* gather(haveGather) (gpugas.h:1553-1619).  Built-in programs only. */
gas_status_t gas_engine_gather(gas_engine *e, int32_t have_gather,
                               void *stream);

/* apply() (gpugas.h:1621-1648).  Built-in programs only. */
gas_status_t gas_engine_apply(gas_engine *e, void *stream);

/* scatterActivate(haveScatter) (gpugas.h:1650-1759): next active set =
 * out-neighbours of the vertices whose apply returned true, ascending id.
 * Program::scatter is not invoked, as in the reference GPU engine. */
gas_status_t gas_engine_scatter_activate(gas_engine *e, int32_t have_scatter,
                                         void *stream);

/* nextIter() (gpugas.h:1761-1772): makes the next active set current and
 * returns its size (synchronises the stream). */
gas_status_t gas_engine_next_iter(gas_engine *e, int32_t *n_active,
                                  void *stream);

/* getResults() (gpugas.h:1778-1787): copies device vertex data back to the
 * host array given to setGraph.  (At the reference's HEAD this body is
 * compiled out; here it does what its comment says.) */
gas_status_t gas_engine_get_results(gas_engine *e, void *stream);

/* run() (gpugas.h:1792-1807): iterate until no vertex is active. */
gas_status_t gas_engine_run(gas_engine *e, int32_t *iterations, void *stream);

/* BFS level used by the built-in BFS apply; mirrors setIterationCount<true>
 * (bfs.cu:83-90). */
gas_status_t gas_engine_set_iteration(gas_engine *e, int32_t level);

/* Device vertex data (nV records) and copies into / out of it from host or
 * device memory (any pointer the CUDA runtime can address), for callers that
 * keep their state resident on the GPU. */
gas_status_t gas_engine_vertex_data_device(gas_engine *e, void **ptr);
gas_status_t gas_engine_upload_vertex_data(gas_engine *e, const void *host,
                                           void *stream);
gas_status_t gas_engine_download_vertex_data(gas_engine *e, void *host,
                                             void *stream);
/* The same copy out without waiting for it: it is queued on stream, and dst
 * must stay valid (and the vertex data unchanged) until it completes.  For
 * callers that overlap the read-back of one run with the next run's work. */
gas_status_t gas_engine_download_vertex_data_async(gas_engine *e, void *dst,
                                                   void *stream);

/* Schedule of the built-in fast runs.  For BFS the pull is the bottom-up
 * level (each unvisited vertex stops at its first in-neighbour of the
 * previous level), and AUTO and LEARNED both take a direction rule: graphs
 * of more than 2^18 vertices Beamer, Asanovic and Patterson's (SC'12;
 * bottom-up once the frontier's out-edges exceed 1/14 of the edges not yet
 * explored, top-down again once it shrinks below V/24 vertices), smaller
 * ones (one cooperative kernel) "bottom-up while the frontier's out-edges
 * exceed E/16". */
typedef enum {
  GAS_SCHED_AUTO = 0,      /* fixed heuristic per iteration                */
  GAS_SCHED_GENERIC = 1,   /* the step-API kernels (pull over active set)  */
  GAS_SCHED_PUSH = 2,      /* push every iteration (SSSP, CC, BFS)         */
  GAS_SCHED_PULL = 3,      /* dense pull every iteration (SSSP, CC, BFS)   */
  GAS_SCHED_ORDERED = 4,   /* generic, but each vertex folds its in-edges  */
                           /* sequentially in CSC order (parity mode)      */
  GAS_SCHED_LEARNED = 5    /* push or pull per iteration from the engine's */
                           /* schedule model (gas_engine_set_schedule_model) */
} gas_schedule_t;

typedef struct {
  int32_t iterations;      /* GAS iterations, counted as run() counts them */
  int32_t push_iters;      /* iterations run with the push schedule        */
  int32_t pull_iters;      /* iterations run with the dense pull schedule  */
  int32_t kernel_launches; /* launches of libgas kernels in the run        */
  int64_t edges_processed; /* edges read by gather / expand kernels        */
  double residual;         /* PageRank: last L1 residual                   */
  int32_t graph_launches;  /* CUDA-graph launches the run took: 1 for the  */
                           /* device loop, 0 with direct launches          */
  int32_t pad;
} gas_run_stats;

/* Runs the built-in program to convergence from the engine's current
 * vertex data and active set (set_active), like run(), with the chosen
 * schedule; the iteration count and final vertex data are identical for
 * every schedule.  Vertex data stays on the device (get_results copies).
 * max_iterations <= 0 selects nV + 2 (BFS, SSSP, CC) or 100000 (PageRank);
 * reaching the cap returns GAS_ERR_ITER_CAP and leaves the engine usable. */
gas_status_t gas_engine_run_schedule(gas_engine *e, gas_schedule_t schedule,
                                     int32_t max_iterations,
                                     gas_run_stats *stats, void *stream);

/* Precision-form PageRank on the engine's graph (no reference counterpart;
 * the reference formula pagerank.cu:62 scaled by 1/N): r0 = 1/N,
 * r'_v = (1-d)/N + d * sum_{u->v} r_u / outdeg(u) with every vertex active
 * every iteration, FP32 gather with two-sum compensation, FP64 L1 residual
 * sum |r' - r|; stops after the first iteration with residual <= tol, on the
 * device (CUDA-graph WHILE loop).  ranks: nV floats, device or host pointer
 * (may be NULL).  Fails with GAS_ERR_ITER_CAP after max_iterations. */
gas_status_t gas_engine_pagerank_precision(gas_engine *e, double damping,
                                           double tol, int32_t max_iterations,
                                           float *ranks, gas_run_stats *stats,
                                           void *stream);

/* One precision-form PageRank step for callers that cannot allocate device
 * memory -- code whose memory pool or arena owns every byte of the device,
 * or a request path that must not call cudaMalloc (it synchronises the device
 * and can fail under fragmentation).  No counterpart in the reference.
 *   rank_out[v] = (1-d)/N + d * sum_{u->v} rank_in[u] / out_degree[u]
 * over a CSC graph in device memory (csc_off[nV+1], csc_src[nE]); *l1_out
 * (device) receives the FP64 residual sum_v |rank_out[v] - rank_in[v]|.
 * All pointers are caller-owned device memory; the kernels' scratch is a
 * fixed file-scope device array of about 6.3 MB.  CUDA loads it (lazy module
 * loading, the default) on a device at the first call there, which is when
 * those 6.3 MB are reserved: make one call first (nV = nE = 0 with a device
 * l1_out will do), or set CUDA_MODULE_LOADING=EAGER, before a pool takes the
 * device; later calls allocate nothing, and the array stays reserved until
 * the process exits.  Graphs with nV + nE > GAS_NOALLOC_MAX_ITEMS return
 * GAS_ERR_TOO_LARGE.  Every call shares that array: calls whose kernels
 * overlap on the GPU race, so issue them on one stream.  Each call looks the
 * array up with the calling thread's device current; make the first call on
 * a device before capturing work into a CUDA graph. */
#define GAS_NOALLOC_MAX_ITEMS (1LL << 29)
gas_status_t gas_pagerank_step_noalloc(int32_t nV, int32_t nE,
                                       const int32_t *csc_off,
                                       const int32_t *csc_src,
                                       const int32_t *out_degree,
                                       const float *rank_in, float *rank_out,
                                       double damping, double *l1_out,
                                       void *stream);

/* Kernel-level measurement of the fast runs.  With profiling on, runs use
 * direct launches (one host read per iteration) and bracket the dominant
 * kernels with CUDA events on the run's stream; times and algorithmic bytes
 * (the bytes the work itself must move: per edge its index, weight and the
 * state it reads; per vertex its offsets and state) accumulate until
 * reset.  No reference counterpart. */
typedef struct {
  double push_ms, pull_ms, pagerank_ms;        /* summed kernel time        */
  int64_t push_bytes, pull_bytes, pagerank_bytes;
  int32_t push_launches, pull_launches, pagerank_launches;
  int32_t pad;
} gas_kernel_profile;

gas_status_t gas_engine_set_profiling(gas_engine *e, int32_t on);
gas_status_t gas_engine_get_profile(gas_engine *e, gas_kernel_profile *out,
                                    int32_t reset);

/* ======================================================================= */
/* Learned parts: MLP, engine traces, schedule head, PageRank warm start.  */
/* No reference counterpart.                                               */
/* ======================================================================= */

#define GAS_MLP_HIDDEN 64    /* two hidden layers of this width, ReLU      */
#define GAS_MLP_MAX_IN 32
#define GAS_MLP_MAX_OUT 2

/* An MLP n_in -> 64 -> 64 -> n_out on the device: FP32 master weights,
 * BF16 copies for every forward pass, FP32 accumulation, Adam state.
 * Flat parameter layout: W1[n_in][64] b1[64] W2[64][64] b2[64]
 * W3[64][n_out] b3[n_out]. */
typedef struct gas_mlp gas_mlp;
gas_status_t gas_mlp_create(int32_t n_in, int32_t n_out, uint64_t seed,
                            gas_mlp **out);
void gas_mlp_destroy(gas_mlp *m);
int64_t gas_mlp_num_params(const gas_mlp *m);
gas_status_t gas_mlp_get_params(const gas_mlp *m, float *host);
gas_status_t gas_mlp_set_params(gas_mlp *m, const float *host);
/* Loss and its gradient for a batch (device pointers): x[batch][n_in];
 * y[batch] class labels (softmax cross-entropy) or t[batch] targets of
 * output 0 (squared error); w[batch] optional sample weights.  The loss is
 * the weighted mean over the batch; grad_host receives all parameters'
 * gradients (may be NULL). */
gas_status_t gas_mlp_gradients(gas_mlp *m, const float *x, const int32_t *y,
                               const float *t, const float *w, int32_t batch,
                               float *grad_host, float *loss_host,
                               void *stream);
/* One Adam step (lr; betas 0.9, 0.999) on the same loss. */
gas_status_t gas_mlp_train_step(gas_mlp *m, const float *x, const int32_t *y,
                                const float *t, const float *w, int32_t batch,
                                float lr, float *loss_host, void *stream);
/* out[n][n_out] = model(x[n][n_in]) with the BF16 weights (device). */
gas_status_t gas_mlp_forward(const gas_mlp *m, const float *x, int32_t n,
                             float *out, void *stream);

/* One iteration of a fast run, as recorded on the device. */
typedef struct {
  int32_t iteration;     /* k                                            */
  int32_t mode;          /* 0 push, 1 dense pull, used for iteration k  */
  int32_t n_queue;       /* |C_{k-1}| restricted to vertices with out-edges */
  int32_t n_edges_out;   /* their out-edges                              */
  int32_t hist[8];       /* their out-degrees: bucket min(7, floor(log2 d)/2) */
  int64_t t_start_ns;    /* %globaltimer when iteration k was scheduled  */
  int64_t t_end_ns;      /* ... when iteration k had finished            */
} gas_trace_record;

#define GAS_SCHED_FEATURES 16
#define GAS_TRACE_CAP 4096

/* Turns per-iteration recording of later fast runs on or off, and copies
 * the last run's records out (n = number written, at most cap). */
gas_status_t gas_engine_set_trace(gas_engine *e, int32_t on);
gas_status_t gas_engine_get_trace(gas_engine *e, gas_trace_record *out,
                                  int32_t cap, int32_t *n);

/* The schedule head's input for iteration rec->iteration: log-scaled
 * frontier size and out-edge count, graph size, frontier shares, degree
 * histogram shares, iteration index, weighted flag (the same function the
 * device loop evaluates). */
void gas_schedule_features(const gas_trace_record *rec, int32_t nV, int64_t nE,
                           int32_t weighted, float *out);

/* GAS_SCHED_LEARNED uses this two-output model (n_in = GAS_SCHED_FEATURES;
 * logit 1 > logit 0 selects the dense pull); NULL removes it.  The model is
 * read when runs launch; it must outlive them. */
gas_status_t gas_engine_set_schedule_model(gas_engine *e, const gas_mlp *m);

/* PageRank warm start: per-vertex features of in- and out-degree (log2 of
 * 1 + degree, over 32) plus graph-level log sizes go through a one-output
 * model (n_in = GAS_WARM_FEATURES) predicting log(N * rank); init receives
 * exp(prediction) / N for every vertex (device or host pointer, nV
 * floats), scaled so that its total equals the mass the fixed point of
 * PageRank with this damping has: (1-d) / (1 - d (1 - delta)), delta the
 * predicted share on vertices without out-edges.  The model is evaluated on
 * a 64 x 64 grid of log-degrees and interpolated bilinearly per vertex. */
#define GAS_WARM_FEATURES 4
gas_status_t gas_engine_pagerank_warm_start(gas_engine *e, const gas_mlp *m,
                                            double damping, float *init,
                                            void *stream);

/* gas_engine_pagerank_precision from a given initial vector (nV floats,
 * device or host; NULL = the uniform 1/N). */
gas_status_t gas_engine_pagerank_precision_from(gas_engine *e, double damping,
                                                double tol,
                                                int32_t max_iterations,
                                                const float *init, float *ranks,
                                                gas_run_stats *stats,
                                                void *stream);

/* Personalized PageRank of one seed on the engine's graph (no reference
 * counterpart): r = (1-d) e_seed + d A^T D^-1 r from r0 = e_seed, with the
 * kernels, compensation and residual of gas_engine_pagerank_precision.
 * The single-instance form of the batched PPR below. */
gas_status_t gas_engine_ppr_precision(gas_engine *e, int32_t seed, double damping,
                                      double tol, int32_t max_iterations,
                                      float *ranks, gas_run_stats *stats,
                                      void *stream);

/* ======================================================================= */
/* Batched engine: many graphs, many BFS sources and personalized-PageRank */
/* seeds per graph, one CUDA-graph launch.  No reference counterpart.      */
/* ======================================================================= */

/* The graphs are stored as one disjoint union graph; graph g's vertex v is
 * union vertex gas_batch_vertex_offset(b, g) + v.  Results are laid out
 * [union vertex][lane]. */
typedef struct gas_batch gas_batch;
gas_status_t gas_batch_create(gas_batch **out);
void gas_batch_destroy(gas_batch *b);
/* Appends a graph (edge list over [0, nV)); graph_id may be NULL. */
gas_status_t gas_batch_add_graph(gas_batch *b, int32_t nV, int64_t nE,
                                 const int32_t *srcs, const int32_t *dsts,
                                 int32_t *graph_id);
/* The same with int32 edge weights in [0, 100000] for the SSSP lanes (the
 * SSSP Program's margin below INT_MAX; weights may be NULL; graphs added
 * without weights weigh 1 per edge). */
gas_status_t gas_batch_add_graph_weighted(gas_batch *b, int32_t nV, int64_t nE,
                                          const int32_t *srcs, const int32_t *dsts,
                                          const int32_t *weights, int32_t *graph_id);
/* Uploads the union graph (CSR + CSC); no graphs can be added afterwards. */
gas_status_t gas_batch_build(gas_batch *b, void *stream);
int32_t gas_batch_num_graphs(const gas_batch *b);
int32_t gas_batch_num_vertices(const gas_batch *b);
int64_t gas_batch_num_edges(const gas_batch *b);
int32_t gas_batch_vertex_offset(const gas_batch *b, int32_t graph);

#define GAS_BATCH_MAX_LANES 32

typedef struct {
  int32_t bfs_lanes;           /* 0..32 BFS sources per graph (0: no BFS)   */
  const int32_t *bfs_sources;  /* [graphs][bfs_lanes] local ids, -1 unused  */
  int32_t ppr_lanes;           /* 0..32 PPR seeds per graph (0: no PPR)     */
  const int32_t *ppr_seeds;    /* [graphs][ppr_lanes] local ids, -1 unused  */
  double damping;              /* PPR damping d in (0, 1)                   */
  double tol;                  /* PPR: stop when every lane's L1 step <= tol */
  int32_t max_bfs_levels;      /* <= 0: union V + 2                         */
  int32_t max_ppr_iterations;  /* <= 0: 1000                                */
  int32_t piece_edges;         /* PPR edges per piece; 0: tuned or 256      */
  int32_t sssp_lanes;          /* 0..32 SSSP sources per graph (0: no SSSP) */
  const int32_t *sssp_sources; /* [graphs][sssp_lanes] local ids, -1 unused */
  int32_t max_sssp_iterations; /* <= 0: union V + 2                         */
} gas_batch_job;

typedef struct {
  int32_t bfs_iterations;      /* push levels run                           */
  int32_t ppr_iterations;
  int64_t bfs_edges;           /* out-edges pushed (lanes of a vertex share) */
  double ppr_residual;         /* largest per-lane L1 step at the end       */
  int32_t piece_edges;         /* piece size the PPR loop used              */
  int32_t kernel_launches;
  int32_t graph_launches;      /* 1, or 0 with GAS_HOST_LOOP=1              */
  int32_t sssp_iterations;     /* SSSP pushes run (the largest lane count)  */
  double ppr_lane_residual[GAS_BATCH_MAX_LANES];
  int64_t sssp_edges;          /* out-edges pushed (lanes of a vertex share) */
  int32_t sssp_lane_iterations[GAS_BATCH_MAX_LANES]; /* pushes per lane: one */
                               /* SSSP from that source runs as many        */
} gas_batch_stats;

/* Runs the job's BFS lanes, its SSSP lanes, then its PPR lanes, as one
 * CUDA-graph launch.  depth_out [V][bfs_lanes] int32 (-1 unreached),
 * dist_out [V][sssp_lanes] int32 (INT_MAX - 100000 unreached) and rank_out
 * [V][ppr_lanes] float may be host or device pointers, or NULL.  A lane
 * whose source or seed is -1 stays unreached / all zero.  GAS_ERR_ITER_CAP
 * when a cap ends a loop (results are then those of the last step). */
gas_status_t gas_batch_run(gas_batch *b, const gas_batch_job *job,
                           int32_t *depth_out, int32_t *dist_out, float *rank_out,
                           gas_batch_stats *stats, void *stream);

/* With profiling on, runs use direct launches and bracket every BFS and
 * SSSP push with CUDA events on the run's stream; push_ms / push_bytes /
 * push_launches accumulate until read with reset != 0.  Algorithmic bytes:
 * BFS, per union edge its index and the destination's visited and next
 * words, per queue entry its edge range and lane mask; SSSP, per union edge
 * its index, weight and destination row, per queue entry its edge range and
 * snapshot row. */
gas_status_t gas_batch_set_profiling(gas_batch *b, int32_t on);
gas_status_t gas_batch_get_profile(gas_batch *b, gas_kernel_profile *out,
                                   int32_t reset);

/* Autotuner: times a few PPR iterations for each piece size in
 * {64, 128, ..., 2048} with ppr_lanes lanes and keeps the fastest for runs
 * whose job says piece_edges = 0. */
gas_status_t gas_batch_tune(gas_batch *b, int32_t ppr_lanes, double damping,
                            int32_t trials, int32_t *piece_edges_out,
                            float *ms_per_iter_out, void *stream);

/* ======================================================================= */
/* Views used by include/gpugas.h to launch its Program-typed kernels.     */
/* ======================================================================= */

/* Device-resident counters of the current frontier (one 64-byte line). */
typedef struct {
  int32_t n_active;        /* |active|                                     */
  int32_t n_edges;         /* sum of in-degree over active (gather work)   */
  int32_t n_scatter_edges; /* sum of out-degree over apply==true vertices  */
  int32_t error;           /* non-zero: a kernel hit an error              */
  int32_t iteration;
  int32_t cond;
  int32_t n_changed;       /* |C_k|: vertices whose apply() returned true  */
  int32_t max_iter;        /* iteration cap of the current device loop     */
  int32_t mode;            /* fast runs: 0 push, 1 dense pull (this iter.) */
  int32_t n_push;          /* fast runs: iterations run with push          */
  int32_t n_pull;          /* fast runs: iterations run with dense pull    */
  int32_t pull_div;        /* AUTO pulls when out-edges(C_k)*pull_div > E  */
  int32_t sched;           /* fast runs: 0 auto, 1 push, 2 pull, 3 learned */
  int32_t push_chunk_log2; /* fast runs: edges per push warp chunk (log2)  */
  int32_t q_heavy;         /* fast runs: queue rows [0, q_heavy) have more */
                           /* out-edges than a thread takes alone          */
  int32_t q_heavy_edges;   /* fast runs: out-edges of those rows           */
  int32_t seen_edges;      /* BFS fast runs: out-edges of the levels before */
                           /* the current queue                           */
  int32_t prev_changed;    /* BFS fast runs: the previous queue's length    */
  int32_t pad[2];
} gas_counters;

typedef struct {
  int32_t nV;
  int32_t nE;
  const int32_t *csc_off;  /* [nV+1] in-edge offsets                       */
  const int32_t *csc_src;  /* [nE]   source of each in-edge                */
  const void *csc_ed;      /* [nE]   edge data in CSC order (may be NULL)  */
  const int32_t *csr_off;  /* [nV+1] out-edge offsets                      */
  const int32_t *csr_dst;  /* [nE]   destination of each out-edge          */
  const void *csr_ed;      /* [nE]   edge data in CSR order (may be NULL)  */
  void *vertex_data;       /* [nV]   device vertex data                    */
  int32_t *active;         /* [nV]   active vertex ids, ascending          */
  int32_t *active_scan;    /* [nV+1] exclusive scan of in-degree over active */
  uint8_t *apply_ret;      /* [nV]   apply() result per active slot       */
  void *slot;              /* [nV]   new vertex data per active slot      */
  void *gather_tmp;        /* [nV]   gather result per active slot        */
  void *tile_first;        /* [tile_cap] gather partials (see gas_device.cuh) */
  void *tile_carry;        /* [tile_cap]                                    */
  int32_t *tile_a0;        /* [tile_cap]                                    */
  int32_t *tile_part;      /* [tile_cap+2] merge-path tile boundaries      */
  int32_t tile_cap;
  int32_t num_sms;         /* SM count of the engine's device              */
  gas_counters *counters;  /* device                                       */
} gas_engine_view;

/* Device pointers of a user engine (valid until the next set_graph). */
gas_status_t gas_engine_view_get(gas_engine *e, gas_engine_view *view);

/* Host-side bookkeeping for user engines: the header tells the engine that
 * its kernels wrote per-slot vertex data (commit pending) or updated the
 * vertex data in place. */
gas_status_t gas_engine_note_applied(gas_engine *e, int32_t wrote_slots);

/* Where set_graph puts the edge arrays (CSC sources, CSR destinations and
 * their edge data; offsets and vertex state stay in HBM).  GAS_EDGES_HOST
 * keeps them in pinned host memory that the kernels read over NVLink-C2C,
 * for graphs whose edges do not fit in HBM -- the role of the reference's
 * host-resident shards (gpugas.h:456-584, 1398-1469).  Applies from the
 * next set_graph. */
typedef enum { GAS_EDGES_DEVICE = 0, GAS_EDGES_HOST = 1 } gas_edge_placement_t;
gas_status_t gas_engine_set_edge_placement(gas_engine *e, gas_edge_placement_t where);

/* Host copies of the engine's CSC and CSR (any pointer may be NULL):
 * csc_off[nV+1], csc_src[nE], csr_off[nV+1], csr_dst[nE], and the edge data
 * in CSC and CSR order (nE records each).  Edges of one row keep their
 * edge-list order (edgeListToCSR / edgeListToCSC, util.cuh:80-121). */
gas_status_t gas_engine_download_graph(gas_engine *e, int32_t *csc_off, int32_t *csc_src,
                                       int32_t *csr_off, int32_t *csr_dst, void *csc_ed,
                                       void *csr_ed, void *stream);

/* Before a user program's scatter kernel (refgas.h:175-196 semantics, which
 * the reference GPU engine skips, gpugas.h:942): publishes the vertex data
 * the last apply wrote, marks the edge data as modified on the device (so
 * that get_results copies it back into the caller's edge array, in edge-list
 * order) and returns the CSC position of every CSR edge (NULL without edge
 * data), through which the kernel keeps the two device copies equal. */
gas_status_t gas_engine_prepare_scatter(gas_engine *e, const int32_t **csr_to_csc,
                                        void *stream);

/* Host copy of the counters (synchronises the stream). */
gas_status_t gas_engine_read_counters(gas_engine *e, gas_counters *out,
                                      void *stream);

/* One iteration's Program-typed kernels of a user engine -- the gather with
 * apply fused into its epilogue, or apply alone -- launched by the caller
 * (include/gpugas.h) on `stream` with grids that do not depend on host-side
 * counts: the call is captured into a CUDA graph, so the kernels must take
 * every size from the device counters. */
typedef gas_status_t (*gas_user_step_fn)(void *ctx, void *stream);

/* run() (gpugas.h:1792-1807) for a user program with the loop on the
 * device: one CUDA-graph launch whose WHILE node runs step(ctx) and then
 * libgas's commit, scatter-activate and compaction kernels until the active
 * set is empty, testing the condition on the device (no host round trip per
 * iteration).  wrote_slots: step writes per-slot vertex data (gather fused
 * with apply, committed after every gather of the iteration has read the
 * old values) rather than updating it in place.  The graph is captured on
 * the first call and reused while (step, ctx, wrote_slots) stay the same,
 * until the next set_graph.  max_iterations <= 0 selects 1,000,000;
 * reaching it returns GAS_ERR_ITER_CAP (the reference loops forever).
 * stats (may be NULL) receives the iteration count run() prints and the
 * launches.  Programs that run Program::scatter on the GPU keep the step
 * loop (their scatter publishes edge data from the host side). */
gas_status_t gas_engine_run_user(gas_engine *e, gas_user_step_fn step, void *ctx,
                                 int32_t wrote_slots, int32_t max_iterations,
                                 gas_run_stats *stats, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GAS_H_ */
