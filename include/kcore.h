/*
 * kcore.h - C ABI of the GB300 k-core peel (libkcore_gb300.so).
 *
 * Drop-in boundary for the reference's single hot path, the level-synchronous
 * peel behind `kcore <edgelist>`.  Every entry point returns 0 (KC_OK) or a
 * negative KC_ERR_* code; none calls exit().  Host buffers are owned by the
 * caller unless a function says otherwise.  Reference citations are paths
 * inside akhlaqueak/KCoreGPU.
 *
 * Threading: a kc_graph / kc_batch is used by one host thread at a time.
 * kc_serve_submit / kc_serve_poll may be called from any thread.
 */
#ifndef KCORE_GB300_H
#define KCORE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (replace chkerr()'s exit(-1), inc/gpu_memory_allocation.h:9-16,
 *      and the device assert() on queue overflow, src/buffer.cc:2) ---- */
#define KC_OK            0
#define KC_ERR_IO       -1   /* file cannot be opened / written                    */
#define KC_ERR_PARSE    -2   /* malformed edge list or serialized cache            */
#define KC_ERR_OOM      -3   /* host or device allocation failed                   */
#define KC_ERR_OVERFLOW -4   /* a device queue would overflow (no trap)            */
#define KC_ERR_TIMEOUT  -5   /* a bounded device wait gave up                      */
#define KC_ERR_CUDA     -6   /* CUDA runtime error                                 */
#define KC_ERR_BUDGET   -7   /* request exceeds the server's HBM budget            */
#define KC_ERR_INVALID  -8   /* bad argument (null pointer, size limit)            */
#define KC_ERR_NODEV    -9   /* no CUDA device                                     */
#define KC_ERR_BUSY    -10   /* server queue full / result not ready               */
#define KC_ERR_CLOSED  -11   /* server already closed                              */

const char* kc_strerror(int code);
/* Message of the last failure on the calling thread (empty when none).          */
const char* kc_last_error(void);
/* SM count, persistent grid size and compute capability of the current device. */
int  kc_device_info(int* sms, int* grid, int* cc_major, int* cc_minor);
/* Page-locked host buffers for the H2D/D2H staging of the calls below.         */
void* kc_host_alloc(size_t bytes);
void  kc_host_free(void* p);

/* ---- host CSR (the reference's Graph arrays, inc/graph.h:7-23) ---- */
typedef struct kc_csr_host {
    uint32_t  V;          /* vertices: max id + 1 (graph.cpp:90-96)              */
    uint32_t  E;          /* arcs = offsets[V] = 2 x undirected edges (graph.cpp:114) */
    uint32_t* offsets;    /* V+1 exclusive prefix of degrees (graph.cpp:110-113)  */
    uint32_t* neighbors;  /* E, ascending within each vertex (graph.cpp:117-122)  */
    uint32_t* degrees;    /* V (graph.cpp:105-108)                                */
} kc_csr_host;

/* Parse modes for the SNAP-style text loader.                                   */
#define KC_PARSE_SNAP       0  /* default: skip lines starting with a letter (graph.cpp:86)
                                  and also '#', '%' and blank lines                 */
#define KC_PARSE_REFERENCE  1  /* byte-for-byte reference stream semantics: a '#'/'%'
                                  line yields s=0 and keeps the previous t
                                  (graph.cpp:86-88); a first line without a
                                  previous t is KC_ERR_PARSE (undefined there)       */

/* Graph::readFile (graph.cpp:58-124): text edge list -> deduplicated, symmetrised
 * CSR with self-loops dropped; V = max id + 1.  Arrays are malloc'ed; free them
 * with kc_csr_free.  Parallel radix CSR build, bytes identical to the reference. */
int  kc_load_edgelist(const char* path, int parse_mode, kc_csr_host* out);

/* Same CSR semantics from an in-memory directed edge array (src[i] -> dst[i]).  */
int  kc_build_csr(const uint32_t* src, const uint32_t* dst, uint64_t n_edges,
                  kc_csr_host* out);

void kc_csr_free(kc_csr_host* csr);

/* Graph::readSerialized / writeSerialized (graph.cpp:9-54): the text CSR cache
 * "V\nE\n" deg[i]"\n"... off[i]" "... nbr[j]" "..., no trailing newline.         */
int  kc_read_serialized(const char* path, kc_csr_host* out);
int  kc_write_serialized(const char* path, const kc_csr_host* csr);

/* Binary CSR sidecar of the serialized cache (no reference counterpart: it
 * cuts load time): "KCCSRBN1", V (uint32), 0 (uint32), E (uint64), then the raw
 * offsets[V+1] and neighbors[E] (uint32, host byte order).  The reader
 * validates sizes, offsets and neighbour ids (KC_ERR_PARSE otherwise).          */
int  kc_write_csr_binary(const char* path, const kc_csr_host* csr);
int  kc_read_csr_binary(const char* path, kc_csr_host* out);

/* Graph::Graph(path) (graph.cpp:142-154): read <cache_dir>/serialized-<basename>
 * when present, else parse the text and write that cache (silently skipped when
 * cache_dir is missing).  cache_dir NULL means "./output/" (inc/common.h:17).
 * Beside the text cache a binary sidecar serialized-<basename>.kcb is written
 * and, unless the text cache is newer, read instead of it.  *from_cache is set
 * to 1 when the text cache was used, 2 for the sidecar (may be NULL).           */
int  kc_load_graph(const char* path, const char* cache_dir, int parse_mode,
                   kc_csr_host* out, int* from_cache);

/* Graph::writeKCoreToDisk (graph.cpp:126-140): JSON '{ "v": c, \n... }\n',
 * vertices with core 0 omitted.                                                 */
int  kc_write_core_json(const char* path, const uint32_t* core, uint32_t V);
/* The verification notebook's "id core" text format, one line per vertex
 * (.ipynb_checkpoints/test-checkpoint.ipynb cell 4).                            */
int  kc_write_core_txt(const char* path, const uint32_t* core, uint32_t V);

/* ---- synthetic graph generators (seeded, deterministic on any host) ---- */
/* R-MAT: n vertices (scale = ceil(log2 n), endpoints >= n redrawn), n_edges
 * directed draws, probabilities a,b,c (d = 1-a-b-c), then a seeded relabel.     */
int  kc_gen_rmat(uint32_t n, uint64_t n_edges, double a, double b, double c,
                 uint64_t seed, uint32_t* src, uint32_t* dst);
/* Chung-Lu power law: weights w_i ~ (i+i0)^(-1/(gamma-1)) scaled to max_w and
 * sum 2*m_target, endpoints by alias sampling, deduplicated and topped up to
 * m_target undirected edges, seeded relabel.  Writes m_target pairs.           */
int  kc_gen_chung_lu(uint32_t n, uint64_t m_target, double gamma, double max_w,
                     uint64_t seed, uint32_t* src, uint32_t* dst);
/* Erdos-Renyi G(n, m): m distinct undirected pairs, no self-loops.              */
int  kc_gen_er(uint32_t n, uint64_t m, uint64_t seed, uint32_t* src, uint32_t* dst);
/* Writes "u\tv\n" lines (no comment or blank lines).                            */
int  kc_write_edgelist(const char* path, const uint32_t* src, const uint32_t* dst,
                       uint64_t n_edges);

/* ---- single-graph peel (replaces kcore(), src/ours.cc:117-160) ---- */
typedef struct kc_stats {
    uint32_t V;
    uint32_t kmax;         /* degeneracy = level-1 at loop exit (ours.cc:151)    */
    uint32_t levels;       /* levels of the reference loop = kmax+1              */
    uint32_t iterations;   /* level iterations run (runs of empty levels skipped) */
    uint32_t blocks;       /* persistent CTAs launched                           */
    uint64_t arcs;         /* offsets[V]                                         */
    uint64_t tasks;        /* hub chunks / spilled vertices pushed to the queue  */
    float    peel_ms;      /* device time of the peel (CUDA events)              */
    float    total_ms;     /* host wall time of the call                         */
    uint32_t method;       /* 1: h-index fixed point, 0: level peel              */
} kc_stats;

typedef struct kc_graph kc_graph;   /* device-resident CSR + peel state         */

/* Pinned H2D upload of a CSR (malloc_graph_gpu_memory, gpu_memory_allocation.cu:4-12).
 * degrees are derived on the device from offsets.                              */
int  kc_graph_upload(const uint32_t* offsets, const uint32_t* neighbors, uint32_t V,
                     kc_graph** g);
/* Use an existing CUDA stream (cudaStream_t passed as void*; NULL = own stream). */
int  kc_graph_set_stream(kc_graph* g, void* stream);
/* Method of this graph's peels: KC_METHOD_AUTO (the process default: the level
 * peel, or what KC_ALGO=peel|hindex names), KC_METHOD_HINDEX (the h-index fixed
 * point, with the level peel after KC_HX_ITERS iterations without convergence)
 * or KC_METHOD_PEEL (the level-synchronous peel).  Same core numbers either
 * way; kc_stats.method reports which one produced them.                        */
#define KC_METHOD_AUTO   0
#define KC_METHOD_HINDEX 1
#define KC_METHOD_PEEL   2
int  kc_graph_set_method(kc_graph* g, uint32_t method);
/* Runs the peel on the device (no host sync).  Results stay on the device.      */
int  kc_graph_peel_async(kc_graph* g);
/* Waits for the last peel, copies core numbers (V uint32, may be NULL) and
 * kmax to the host (get_results_from_gpu, gpu_memory_allocation.cu:14-16).       */
int  kc_graph_fetch(kc_graph* g, uint32_t* core_out, uint32_t* kmax, kc_stats* st);
/* kc_graph_peel_async + kc_graph_fetch.                                          */
int  kc_peel(kc_graph* g, uint32_t* core_out, uint32_t* kmax, kc_stats* st);
/* Peel order (vertices by level; the kcore-global-buffer glBuffer, KCore.h:80)
 * and k-shell offsets (cShellOffsets, KCore.h:266): order_out[V],
 * shell_offsets_out[kmax+2].  Runs a peel that records the order.                */
int  kc_degeneracy_order(kc_graph* g, uint32_t* order_out,
                         uint32_t* shell_offsets_out, uint32_t shell_cap,
                         uint32_t* kmax);
/* Tracing: runs a peel that records per-level device timestamps (ns of
 * %globaltimer) and counters, 8 words per level iteration: start, CTA 0
 * arrival, announced complete, CTA 0 saw completion, vertices peeled so far,
 * last CTA arrival, walk rounds, 16-byte adjacency quads walked.  Levels run by
 * the one-CTA tail kernel have start, end (words 1, 2, 3, 5), peeled, rounds
 * and quads; the first of them keeps the hand-off's times in words 1, 2, 5
 * (both barriers passed, CTA 0's fill done) and starts at the tail kernel's
 * entry; grid levels have 0 rounds and quads.  out holds level_cap*8 words;
 * *levels = iterations run.  (The reference's per-level trace is a
 * commented-out cout, src/ours.cc:148.)                                          */
int  kc_graph_trace(kc_graph* g, uint64_t* out, uint32_t level_cap, uint32_t* levels);
/* Device pointers of the resident CSR/core arrays (for zero-copy consumers).     */
int  kc_graph_device_ptrs(kc_graph* g, const uint32_t** d_offsets,
                          const uint32_t** d_neighbors, uint32_t** d_core);
void kc_graph_free(kc_graph* g);

/* The autotuner's settings for a graph (no reference counterpart; the
 * reference's are compile-time constants, inc/common.h:4-12).  Chosen at upload
 * (kc_graph_upload, kc_peel_csr) from the degree distribution sampled from the
 * host offsets; none of them changes a result.                                 */
typedef struct kc_tuning {
    uint32_t hub_arcs;       /* vertices with more arcs are split into queued tasks  */
    uint32_t chunk_arcs;     /* arcs per queued task (64..256)                       */
    uint32_t local_budget;   /* arcs a warp's cascade list holds before queueing     */
    uint32_t tail_v;         /* survivors at which the one-CTA tail takes over (0: never) */
    uint32_t grid;           /* persistent CTAs (0: one per SM)                      */
} kc_tuning;
int  kc_autotune(const uint32_t* offsets, uint32_t V, kc_tuning* out);

/* One-shot: host CSR in, host core numbers out (cached device buffers per
 * device; pinned host arrays upload fastest).  The CSR is checked on the device
 * after the upload, before the peel reads it (KC_ERR_INVALID).  kmax as the
 * reference computes it (0xFFFFFFFF for V=0).  Replaces kcore(Graph&),
 * src/ours.cc:117-160, with the core numbers returned.                          */
int  kc_peel_csr(const uint32_t* offsets, const uint32_t* neighbors, uint32_t V,
                 uint32_t* core_out, uint32_t* kmax);

/* ---- batched peel: many independent graphs in one persistent launch ----
 * No reference counterpart (the reference peels one graph per process).  The
 * graphs are packed as one segmented CSR with graph-local uint32 ids and
 * offsets and 64-bit per-graph bases.                                          */
typedef struct kc_segcsr {
    uint32_t        ngraphs;
    const uint64_t* vbase;      /* ngraphs+1: first vertex of graph g (prefix of V_g)  */
    const uint64_t* abase;      /* ngraphs+1: first arc of graph g (prefix of E_g)     */
    const uint32_t* offsets;    /* graph g: V_g+1 local offsets at vbase[g]+g          */
    const uint32_t* neighbors;  /* graph g: E_g local neighbour ids at abase[g]        */
} kc_segcsr;

typedef struct kc_segcsr_host {   /* library-owned segmented CSR (kc_gen_batch)     */
    uint32_t  ngraphs;
    uint64_t* vbase;
    uint64_t* abase;
    uint32_t* offsets;
    uint32_t* neighbors;
} kc_segcsr_host;

typedef struct kc_batch_stats {
    uint32_t ngraphs;
    uint32_t giants;      /* graphs the autotuner sent to the grid-wide peel      */
    uint32_t blocks;      /* CTAs of the batched kernel                           */
    uint32_t qcap;        /* per-CTA queue entries (largest batched graph)        */
    uint64_t V_total;
    uint64_t arcs_total;
    float    peel_ms;     /* device time of the whole batch (CUDA events)         */
} kc_batch_stats;

typedef struct kc_batch kc_batch;

/* Uploads a segmented CSR and runs the autotuner: per-graph cost from the
 * degree histogram (V, E, max degree, h-index), largest-first schedule over the
 * CTAs, graphs too large for one CTA routed to the grid-wide peel, per-CTA
 * queue size and CTAs per SM.                                                  */
int  kc_batch_upload(const kc_segcsr* graphs, kc_batch** b);
int  kc_batch_set_stream(kc_batch* b, void* stream);
/* One persistent launch over all graphs (plus one grid-wide launch per giant). */
int  kc_batch_peel_async(kc_batch* b);
/* Waits; copies core numbers (sum of V_g, graph g at vbase[g]) and per-graph
 * kmax (ngraphs) to the host; either may be NULL.                             */
int  kc_batch_fetch(kc_batch* b, uint32_t* core_out, uint32_t* kmax_out, kc_batch_stats* st);
/* Baseline: the plain single-graph peel launched once per graph, back to back
 * on the stream; results land in the same buffers.  *ms_out = device time.    */
int  kc_batch_peel_per_graph(kc_batch* b, float* ms_out);
/* The autotuner's plan: giants first, then the batched schedule (ngraphs ids). */
int  kc_batch_plan(kc_batch* b, uint32_t* schedule_out, uint32_t* ngiants, uint32_t* qcap,
                   uint32_t* blocks);
void kc_batch_free(kc_batch* b);
/* One-shot: upload, peel, fetch, free.                                         */
int  kc_batch_peel(const kc_segcsr* graphs, uint32_t* core_out, uint32_t* kmax_out,
                   kc_batch_stats* st);
/* Batch generator: graph g uses seed seed_base+g, n ~ log-uniform[nmin,nmax],
 * average degree 2m/n ~ U[dmin,dmax]; even g Erdos-Renyi G(n,m), odd g R-MAT
 * (a,b,c) with m draws; each graph deduplicated/symmetrised as kc_build_csr.   */
int  kc_gen_batch(uint32_t ngraphs, uint64_t seed_base, uint32_t nmin, uint32_t nmax,
                  double dmin, double dmax, double a, double b, double c, kc_segcsr_host* out);
void kc_segcsr_free(kc_segcsr_host* s);

/* ---- served peel: continuous batching of k-core requests ----
 * No reference counterpart.  A request loop admits submitted graphs against an
 * HBM budget (first come, first served), uploads them, and hands them to a
 * persistent serve kernel that keeps running while requests flow: small graphs
 * are peeled by one CTA each, large ones by a gang of CTAs (one CTA per
 * gang_arcs arcs, up to max_gang), and requests that arrive while others run
 * start as soon as CTAs and memory free up.  submit/poll/wait are thread-safe. */
typedef struct kc_serve_cfg {
    uint64_t hbm_budget_bytes;   /* device memory the admitted requests may hold (0: 64 GiB) */
    uint32_t ring_slots;         /* max requests admitted at once (0: 1024)              */
    uint32_t gang_arcs;          /* arcs per gang CTA (0: 2^19)                           */
    uint32_t max_gang;           /* largest gang (0: every CTA of the kernel)             */
    uint32_t small_vertices;     /* largest graph one CTA may peel alone (0: 2^18)        */
} kc_serve_cfg;

typedef struct kc_serve_timing {
    double   queue_us;           /* submit -> admitted                                   */
    double   latency_us;         /* submit -> core numbers on the host                   */
    uint32_t gang;               /* CTAs that peeled it                                  */
    uint32_t iterations;         /* level iterations run                                 */
    double   copy_in_us;         /* device clock: job start -> CSR in device memory      */
    double   peel_us;            /* device clock: CSR in -> peel done                    */
    double   copy_out_us;        /* device clock: peel done -> result published          */
} kc_serve_timing;

typedef struct kc_serve_stats {
    uint64_t submitted;
    uint64_t completed;
    uint64_t in_use;             /* device bytes held by admitted requests now           */
    uint64_t peak_in_use;
    uint32_t pending;
    uint32_t inflight;
    uint32_t blocks;             /* CTAs of the serve kernel                             */
    uint32_t direct;             /* 1: jobs copy their CSR and result through the device's
                                    access to pageable host memory, 0: pinned staging       */
} kc_serve_stats;

typedef struct kc_server kc_server;

int  kc_serve_open(const kc_serve_cfg* cfg, kc_server** s);   /* cfg may be NULL    */
/* Queues a CSR (host arrays that must stay valid until the request completes);
 * the core numbers are written to core_out (V entries).  KC_ERR_BUDGET when the
 * request alone exceeds the budget, KC_ERR_CLOSED after kc_serve_close,
 * KC_ERR_INVALID for offsets that do not start at 0 or decrease.  A neighbour
 * id >= V fails the request with KC_ERR_INVALID (checked while it is copied). */
int  kc_serve_submit(kc_server* s, const uint32_t* offsets, const uint32_t* neighbors,
                     uint32_t V, uint32_t* core_out, uint64_t* request_id);
/* KC_OK (and forgets the request) once core_out holds the result, KC_ERR_BUSY
 * while it is still queued or running.                                         */
int  kc_serve_poll(kc_server* s, uint64_t request_id, uint32_t* kmax, kc_serve_timing* t);
int  kc_serve_wait(kc_server* s, uint64_t request_id, uint32_t* kmax, kc_serve_timing* t,
                   double timeout_s);
int  kc_serve_stats_get(kc_server* s, kc_serve_stats* st);
/* Read-only diagnostic snapshot of the server's device and host state (see
 * kc_serve.cu for the word layout); n = capacity of out (>= 10).              */
int  kc_serve_debug(kc_server* s, uint64_t* out, uint32_t n);
/* Finishes the queued requests, stops the kernel and frees everything.        */
int  kc_serve_close(kc_server* s);

/* ---- allocation-free single-graph peel (no counterpart in the reference) ----
 * For callers that cannot call cudaMalloc: a plugin whose host application owns
 * all device memory through its own pool, or a latency-critical loop where an
 * allocation would add allocator latency and device-wide synchronisation.  The
 * caller passes device buffers: offsets (V+1), neighbors (n_arcs), core_out
 * (V); kmax is copied to the host pointer kmax_out (may be NULL).  The call
 * allocates nothing: its scratch is one static device array sized for
 * V <= KC_NOALLOC_MAX_V and n_arcs <= KC_NOALLOC_MAX_ARCS (larger graphs are
 * rejected with KC_ERR_INVALID), held by every GPU that loads the library until
 * exit.  The first call on a device resolves that array's address; make it
 * before any stream capture.  All calls on a device share the array: calls
 * that overlap on the GPU race, so serialise them.  Returns when done.        */
#define KC_NOALLOC_MAX_V     524288u
#define KC_NOALLOC_MAX_ARCS  8388608u
int  kc_peel_noalloc(const uint32_t* d_offsets, const uint32_t* d_neighbors, uint32_t V,
                     uint32_t n_arcs, uint32_t* d_core_out, uint32_t* kmax_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* KCORE_GB300_H */
