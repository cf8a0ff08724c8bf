/*
 * grg.h -- C ABI of the GB300 CFL-reachability closure engine (libgrg.so).
 *
 * Drop-in boundary for the hot path of Graspan-G. The reference's boundary is
 * the C++-linkage API in src/kernel.h:115-129 plus the globals
 * selectedDevice/numLabels/numVars (src/kernel.h:22-24) and the CUDA calls the
 * host makes directly (device selection src/main.cpp:30-58, pool read-back
 * src/main.cpp:477-483, cudaFree src/main.cpp:903). That API is a
 * non-reentrant singleton; this one carries an explicit context, returns an
 * int status instead of exit(-1) (src/kernel.h:53-58), uses 64-bit sizes, and
 * takes plain pointers and sizes only.
 *
 * Threading: a context is used by one host thread at a time. All device work
 * of a context is issued on its stream (grg_set_stream). Contexts share no
 * device state: each passes its own grammar to every kernel it launches, so
 * different contexts (with different grammars) can be used from different
 * threads and streams at the same time.
 */
#ifndef GRG_H
#define GRG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define GRG_OK 0
#define GRG_NEED_REPARTITION 1   /* partition does not fit its budget (the reference's r=true, src/kernel.cu:65-76) */
#define GRG_PAUSED 2             /* grg_part_run stopped at its run budget; call it again to continue */
#define GRG_E_ARG (-1)           /* invalid argument */
#define GRG_E_CUDA (-2)          /* CUDA runtime error (see grg_last_error) */
#define GRG_E_NOMEM (-3)         /* device or host memory exhausted */
#define GRG_E_FILTER (-4)        /* filter_flag=1 on a grammar where it is schedule-dependent */
#define GRG_E_IO (-5)            /* file could not be read or is malformed */
#define GRG_E_LABEL (-6)         /* graph label not present in the grammar */
#define GRG_E_RANGE (-7)         /* vertex id >= numVars, too many rules or labels */
#define GRG_E_STATE (-8)         /* call made out of order */
#define GRG_E_NODEV (-9)         /* no CUDA device */
#define GRG_E_INTERNAL (-10)     /* a bounded internal loop ran out (table growth that did not
                                    converge) or a consistency check failed; not a CUDA error */

#define GRG_MAX_RULES 64
#define GRG_MAX_LABELS 63        /* label ids 1..63; each may also get a reverse-index slot */
#define GRG_NAME_LEN 64
#define GRG_ELEM_IDS 192         /* ids per element: 6 x 32-bit bitmap words (src/kernel.h:32-33) */

typedef struct grg_ctx grg_ctx;

/* Per-run statistics. Work counters are in the reference's element unit
 * (32 bytes per 192-id element, src/kernel.h:32-44). */
typedef struct grg_stats {
    uint64_t total_edges;          /* FINAL NUM EDGES (src/main.cpp:909-917) */
    uint64_t rounds;               /* semi-naive rounds to the fixpoint */
    uint64_t delta_elems;          /* delta elements joined (sum over rounds) */
    uint64_t left_elems;           /* left-operand elements read by binary joins */
    uint64_t right_elems;          /* right-operand elements read by binary joins */
    uint64_t out_elems;            /* elements written as new deltas */
    uint64_t retry_records;        /* delta records re-run after a table grew */
    uint64_t grow_rows;            /* rows whose table grew */
    uint64_t pool_elems_used;      /* pool slots in use at the end */
    uint64_t pool_elems_cap;       /* pool slots allocated */
    double closure_ms;             /* device time from resident graph to fixpoint known */
    double join_ms;                /* sum of join-kernel durations (when kernel timing is on) */
    uint64_t join_launches;        /* join-kernel launches (first pass + retries) */
    uint64_t kernel_launches;      /* all kernel launches of the closure */
    uint64_t join_phase_cycles[5]; /* join-kernel cycles per phase (record load, unary,
                                      binary join, flush, retry list) when built with
                                      -DGRG_PHASE_TIMERS; 0 otherwise */
    uint64_t window_out_elems;     /* right-hand items the join ORed into its hash
                                      accumulator: beyond the record's dense window, or of a
                                      run of records left without a window slot */
    uint64_t wide_window;          /* 1 = the closure ended on the wide join window */
    double gather_ms;              /* time of the rounds' gathers (when kernel timing is on) */
    uint64_t window_tuned;         /* how the join window was chosen: 0 fixed by grg_set_join_window,
                                      1 measured in this closure, 2 taken from the tuning cache */
    double window_trial_ms[2];     /* the measured trial passes (narrow, wide) when window_tuned = 1 */
    uint64_t column_labels;        /* labels stored by destination in this closure (bit l-1 = label l;
                                      grg_set_layout); their joins are pushes, so right_elems then
                                      counts the edges of C the pushes walked */
    uint64_t push_flat;            /* 1 = pushes dealt the edges of C over the lanes, 0 = one lane per
                                      record (grg_set_push; 0 when nothing is pushed) */
    uint64_t push_tuned;           /* how the push kernel was chosen: 0 fixed, 1 measured in this
                                      closure, 2 taken from the tuning cache */
    double push_trial_ms[2];       /* the measured trial passes (one lane per record, flattened) */
    uint64_t join_elements;        /* 1 = k_join read CSR-copied right-hand rows as whole table
                                      elements, 0 = as destination ids (grg_set_join_items) */
    double items_trial_ms[2];      /* the measured trial passes (ids, elements) when tuned */
    uint64_t window_noslot_items;  /* of window_out_elems: items of a run of records that drew
                                      no window slot (0 unless built with -DGRG_RUN_PASSES=0) */
    uint64_t candidates;           /* elements the joins wrote as candidates for k_apply
                                      (joins insert directly when there is no buffer) */
    uint64_t join_inserts;         /* element inserts the joins made themselves (unary rules,
                                      and flushes without a candidate buffer) */
    uint64_t direct_inserts;       /* 1 = the joins inserted their elements themselves (the
                                      default for grammars with a derivable right-hand label;
                                      environment GRG_DIRECT_INSERTS=0 / 1 overrides), 0 = they
                                      wrote candidates that k_apply inserted */
} grg_stats;

/* Error text of a status code, and the last detailed message of a context. */
const char *grg_error_string(int status);
const char *grg_last_error(const grg_ctx *ctx);

/* Create a context on a device; device < 0 selects the device with the most
 * SMs. Replaces checkGPUConfiguration (src/main.cpp:30-58). */
int grg_create(grg_ctx **ctx, int device);
/* Free every device and host resource of the context (src/main.cpp:903). */
void grg_destroy(grg_ctx *ctx);
/* Selected device ordinal (the reference's global selectedDevice, src/kernel.h:22). */
int grg_device(const grg_ctx *ctx);
/* Issue all work of the context on this cudaStream_t (NULL = the context's own stream). */
int grg_set_stream(grg_ctx *ctx, void *stream);
/* Measure the join pass of every round (adds a little host overhead): CUDA
 * events around host-driven passes, the global nanosecond timer inside
 * device-driven rounds. */
int grg_set_kernel_timing(grg_ctx *ctx, int on);
/* Device-driven rounds (default on; environment GRG_DEVICE_ROUNDS=0 turns the
 * default off): after the first round, grg_closure replays one round from a
 * CUDA graph with a WHILE node until the fixpoint or until a round needs the
 * host (table growth, buffer room), instead of launching and waiting per
 * round. The results are identical either way. */
int grg_set_device_rounds(grg_ctx *ctx, int on);
/* Join window: the join ORs right-hand elements into a dense window per run of
 * a row's records, of 12 elements (mode 1) or 8 (mode 0); elements outside it
 * go to a small shared-memory hash. Mode 2 (the default) tunes the choice: the
 * closure's input is keyed by its grammar, filter, vertex count and the
 * distribution of its table sizes (elements per label and row, log2 buckets);
 * the first closure of a key whose first round is large times a slice of that
 * round's join in each window and keeps the faster (the wide window unless
 * narrow wins by 10% on a trial of at least 0.25 ms), and later closures with
 * the key reuse the choice (a process-wide cache). Mode 3 measures again even
 * when the key is cached, and updates the cache. Environment
 * GRG_JOIN_WINDOW=narrow / wide / tuned selects the default. Results are
 * identical in every mode. */
int grg_set_join_window(grg_ctx *ctx, int mode);
/* Right-hand items of labels that have a CSR copy (never derived, read as a
 * binary rule's second symbol): mode 0 reads destination ids (4 bytes each,
 * one window bit per id), mode 1 reads the label's table elements (32 bytes
 * each, up to 192 ids ORed at once: fewer items to deal over the lanes when a
 * row's ids share elements). Mode 2 (the default) tunes the choice together
 * with the join window (see grg_set_join_window), mode 3 re-measures.
 * Environment GRG_JOIN_ITEMS=ids / elements selects the default. Results are
 * identical. */
int grg_set_join_items(grg_ctx *ctx, int mode);

/* Storage layout of the next graph loaded with grg_load_edges (or batch):
 * mode 0 (the default) stores every label by source, as the reference does;
 * mode 1 (environment GRG_LAYOUT=columns) stores a label by destination -- the table of (label, j) holds the sources i of edges
 * (i, j) -- when the grammar allows it: the label is derived, every binary rule
 * A ::= B C that involves it has a C that is never derived and stores A and B
 * alike, and no old-left join reads it. A rule A ::= B C is then joined by
 * pushing each new element of B's column k (up to 192 sources) whole into A's
 * column j for every edge (k, j) of C, instead of visiting every
 * source-intermediate pair (the dataflow grammar N ::= N e | e is the case
 * this is for). On that grammar's 2M-vertex closure the pushes cost what the
 * source-row join costs but the delta elements by destination are 2.4x as many
 * (sources reach a vertex from several blocks), so the gather doubles and
 * mode 0 is faster; mode 1 stays for inputs where columns are denser.
 * Results are identical either way; the entry points that read rows by source
 * (grg_get_degree, grg_export_elements, grg_range_counts, grg_range_reach,
 * grg_export_csr5) first turn destination-stored labels into rows by source
 * on the device, once per loaded graph. grg_part_create and grg_part_restore
 * set mode 0 on their context. */
int grg_set_layout(grg_ctx *ctx, int mode);
/* Push kernel for destination-stored labels: mode 0 gives each delta record
 * one lane, which walks its row of C alone; mode 1 deals the edges of the
 * rows of C of a warp's 32 records over its lanes (a long row then does not
 * hold the warp while other lanes idle); mode 2 (the default) tunes the choice
 * per degree key like the join window (the first closure of a key times both on
 * a slice of its first large round and keeps the faster, later closures take it
 * from the process-wide cache); mode 3 measures again. Environment
 * GRG_PUSH=lane / flat / tuned selects the default. Results are identical. */
int grg_set_push(grg_ctx *ctx, int mode);

/* Grammar: rules[3*i+{0,1,2}] = LHS, RHS1, RHS2 label ids (1-based, 0 = absent),
 * num_labels = number of distinct labels. Replaces transferRules
 * (src/kernel.cu:22-31), which takes rules from readAndTransferRules
 * (src/main.cpp:69-97). The caller keeps ownership of rules. */
int grg_transfer_rules(grg_ctx *ctx, int num_rules, const int *rules, int num_labels);
/* The context's grammar as given to grg_transfer_rules (rules: 3*GRG_MAX_RULES ints). */
int grg_get_rules(const grg_ctx *ctx, int *num_rules, int *rules, int *num_labels);

/* Reserve the element pool: pool_bytes of device memory for 32-byte elements
 * plus their delta bitmaps (0 = size it from the free device memory).
 * Replaces allocateElementPool (src/kernel.cu:33-40). The pool grows on
 * demand while device memory lasts. */
int grg_allocate_pool(grg_ctx *ctx, uint64_t pool_bytes);

/* Load the labelled graph: num_edges edges (src[i], dst[i], label[i]) over
 * vertices [0, num_vars), labels 1..num_labels. on_device != 0 means the three
 * arrays are device pointers; otherwise they are host memory and are copied.
 * Edges need not be sorted; duplicates collapse. Replaces getGraphInfo +
 * readEdges + createGraph + transferElements (src/main.cpp:106-333,
 * src/kernel.cu:42-52); the pool image is built on the device. */
int grg_load_edges(grg_ctx *ctx, uint32_t num_vars, uint64_t num_edges, const uint32_t *src,
                   const uint32_t *dst, const uint8_t *label, int on_device);

/* Run the semi-naive closure to its fixpoint. filter = the reference's
 * filter_flag (src/main.cpp:890,894): 0 = every rule, 1 = the dataflow
 * optimisation (unary rules and old-left joins skipped; refused with
 * GRG_E_FILTER when a binary rule's second symbol is derivable). Replaces the
 * superstep driver precomputation/run_computation (src/main.cpp:764-858,
 * 892-906) with spagpu_s/spagpu_b/spagpu/mergeAndDiff
 * (src/kernel.cu:466-780, 943-985). stats may be NULL. */
int grg_closure(grg_ctx *ctx, uint32_t filter, grg_stats *stats);

/* grg_closure for a graph loaded with grg_load_elements: the round-1 deltas
 * are the records marked at the load, and every element that gains bits
 * during this closure gets stamp run_stamp (0 = stamps unchanged). One call
 * closes the loaded vertex ranges together, like one spagpu_s/spagpu_b/spagpu
 * pass over a partition or a pair of partitions (src/kernel.cu:466-780). */
int grg_closure_ex(grg_ctx *ctx, uint32_t filter, uint32_t run_stamp, grg_stats *stats);

/* Per-label closure edge counts: counts[l-1] for label l (num_labels values). */
int grg_label_counts(grg_ctx *ctx, uint64_t *counts);

/* Degree table of vertices [first_var, last_var] like getDegree
 * (src/kernel.cu:818-839): degree[v - first_var + n*c] for n = last_var -
 * first_var + 1 and column c: 0 = edges (popcount over all labels), 3 =
 * elements (192-id elements over all labels); columns 1,2,4,5 (delta and tmp
 * regions of the reference) are 0 after the fixpoint. */
int grg_get_degree(grg_ctx *ctx, uint32_t first_var, uint32_t last_var, uint32_t *degree);

/* Order-independent 64-bit hash of the closure edge set
 * (sum over edges of a splitmix64-based hash of (label, src, dst)). */
int grg_set_hash(grg_ctx *ctx, uint64_t *hash);

/* Copy closure edges to host arrays (unordered). *num_out = total edges; at
 * most cap are written. */
int grg_export_edges(grg_ctx *ctx, uint64_t cap, uint32_t *src, uint32_t *dst, uint8_t *label,
                     uint64_t *num_out);

/* ---- Element images: the pool contents of a vertex range, for out-of-core
 * schedules. An image is num_elems records of 8 uint32 words (words 0-5: bitmap
 * of 192 destination ids base*192.., word 6: label << 25 | base, word 7: source
 * vertex) plus one uint32 stamp per record. Replaces transferElements
 * (src/kernel.cu:42-52) and transferBackElements (src/main.cpp:477-483),
 * whose images are raw pool words with linked-list heads. */

/* Load a graph over [0, num_vars) from element records (no epsilon rules are
 * applied: images already hold their epsilon edges). Records whose stamp is
 * above mark_after are the deltas of round 1 of the next grg_closure_ex.
 * Records must be distinct per (label, source, base); out-of-range or repeated
 * records fail with GRG_E_ARG. on_device as for grg_load_edges. */
int grg_load_elements(grg_ctx *ctx, uint32_t num_vars, uint64_t num_elems, const uint32_t *elems,
                      const uint32_t *stamps, uint32_t mark_after, int on_device);
/* Image of source vertices [v_begin, v_end), all labels, into HOST arrays of
 * cap records (8 words each) and cap stamps. *num_out = records in the range;
 * GRG_E_RANGE (nothing written) when that exceeds cap. */
int grg_export_elements(grg_ctx *ctx, uint32_t v_begin, uint32_t v_end, uint64_t cap, uint32_t *elems,
                        uint32_t *stamps, uint64_t *num_out);
/* Per-label edge counts (num_labels values) and edge-set hash (may be NULL;
 * same hash terms as grg_set_hash) of the rows [v_begin, v_end). */
int grg_range_counts(grg_ctx *ctx, uint32_t v_begin, uint32_t v_end, uint64_t *counts, uint64_t *hash);
/* Partitions that rows [v_begin, v_end) reach: reach[p] = 1 (num_parts
 * values) when an edge of a label in label_mask (bit l-1 = label l) from those
 * rows may end in [bounds[p], bounds[p+1]) (bounds: num_parts+1 non-decreasing
 * vertex ids). May report a partition too many, never one too few. A pair
 * of partitions neither of which reaches the other has no join across them
 * (the reference's data-dependence manager idea, src/ddm.cpp:9-132). */
int grg_range_reach(grg_ctx *ctx, uint32_t v_begin, uint32_t v_end, uint64_t label_mask, uint32_t num_parts,
                    const uint32_t *bounds, uint8_t *reach);
/* Cap the element pool at pool_bytes of device memory (0 = no cap): a load or
 * closure that needs more fails with GRG_E_NOMEM instead of growing the pool.
 * A pool already larger is freed (the loaded graph is dropped). */
int grg_set_pool_limit(grg_ctx *ctx, uint64_t pool_bytes);

/* ---- The reference's compressed edge stream: its CSR spill format
 * (COMPRESSED=1), written by storeElements_c / elements2Edges
 * (src/main.cpp:510-596) and read by readElements_c / edges2Elements
 * (src/main.cpp:335-445, 364-445). For each source vertex in order, for each
 * label 1..L, the vertex's destinations ascending, 5 bytes per edge: the
 * destination as a little-endian uint32, then the label id (uint8). The row
 * lengths (edges per source vertex) travel beside it, as the reference keeps
 * them in degree[] (src/main.cpp:541-548). */

/* Rows [v_begin, v_end) of the loaded graph into HOST buffers: edges (cap x 5
 * bytes) and degree (v_end - v_begin values). *num_edges = the stream's length
 * in edges; GRG_E_RANGE (nothing written) when that exceeds cap, so cap = 0
 * asks for the size. Converted on the device (records sorted by row, label,
 * base), in row pieces that fit half of the free device memory. */
int grg_export_csr5(grg_ctx *ctx, uint32_t v_begin, uint32_t v_end, uint64_t cap, uint8_t *edges,
                    uint32_t *degree, uint64_t *num_edges);
/* Load a graph over [0, num_vars) from a stream of num_edges edges whose source
 * rows are [v_begin, v_end) with row lengths degree (v_end - v_begin values),
 * as readElements_c reloads a spilled partition: the stream becomes element
 * records on the device (consecutive edges of a row with one label and 192-id
 * base share a record), loaded as grg_load_elements loads them with every
 * record a delta of round 1; epsilon rules are not applied (a spilled image
 * holds its epsilon edges). Each row's edges must be in the stream's order
 * (label, then destination): a record that repeats fails with GRG_E_ARG, as do
 * lengths that do not add up to num_edges; labels outside 1..L fail with
 * GRG_E_LABEL, destinations >= num_vars with GRG_E_RANGE. on_device as for
 * grg_load_edges (both arrays); a host stream goes to the device in row pieces
 * of at most a quarter of the free device memory. */
int grg_load_csr5(grg_ctx *ctx, uint32_t num_vars, uint32_t v_begin, uint32_t v_end, const uint32_t *degree,
                  uint64_t num_edges, const uint8_t *edges, int on_device);

/* ---- Out-of-core closure over vertex-range partitions (host scheduler on
 * the calls above). Replaces the reference's partitioned driver: partition
 * set-up (src/main.cpp:141-175), precomputation / run_computation supersteps
 * over partition pairs (src/main.cpp:764-858), repartitioning
 * (src/main.cpp:633-762) and the partition spill files (src/main.cpp:447-456,
 * 602-610). Partition images live in host memory; the device holds one pair
 * of partitions (or, when every binary rule's second symbol is never derived,
 * the static labels of the whole graph plus one partition) at a time, within
 * the context's pool limit (grg_set_pool_limit). A partition whose run does
 * not fit is split in two at its median element and the run is repeated. */
typedef struct grg_part grg_part;
typedef struct {
    uint64_t total_edges;     /* closure edges, all labels */
    uint32_t num_parts;       /* partitions at the end (after splits) */
    uint32_t schedule;        /* 0 = stream (independent rows), 1 = pairs */
    uint64_t supersteps;      /* sweeps over the partition pairs (pairs schedule) */
    uint64_t runs;            /* closures run on the device */
    uint64_t skipped;         /* pairs skipped: nothing new since their last run */
    uint64_t splits;          /* partitions split because a run did not fit */
    uint64_t rounds;          /* semi-naive rounds over all runs */
    uint64_t h2d_bytes;       /* image bytes loaded to the device */
    uint64_t d2h_bytes;       /* image bytes read back */
    double ms;                /* wall time of grg_part_run */
    double stage_ms;          /* of which: assembling run inputs in host memory */
    double load_ms;           /*           loading them on the device (grg_load_elements) */
    double closure_ms;        /*           closures (grg_closure_ex) */
    double export_ms;         /*           reading images back (grg_export_elements) */
    double count_ms;          /*           per-partition counts and reach sets */
    uint64_t prefetched;      /* runs whose input a helper thread assembled and copied to the device
                                 (on a copy stream) while the run before computed */
    uint64_t prefetch_hits;   /* of those, runs that loaded the prepared input (the others were
                                 superseded by a run the schedule had not foreseen) */
} grg_part_stats;

/* A partitioned graph over [0, num_vars) on context ctx (which holds the
 * grammar, from grg_transfer_rules, and the pool limit), split into num_parts
 * vertex ranges of equal size (at least 1 vertex each). */
int grg_part_create(grg_part **part, grg_ctx *ctx, uint32_t num_vars, uint32_t num_parts);
void grg_part_destroy(grg_part *part);
/* Input edges (HOST arrays) with the conventions of grg_load_edges; builds the
 * partition images on the device one partition at a time. */
int grg_part_load_edges(grg_part *part, uint64_t num_edges, const uint32_t *src, const uint32_t *dst,
                        const uint8_t *label);
/* Close the graph (filter as for grg_closure). stats may be NULL; they count
 * this call's work. GRG_PAUSED when the run budget stopped it. */
int grg_part_run(grg_part *part, uint32_t filter, grg_part_stats *stats);
/* Per-label closure edge counts (num_labels values) and the edge-set hash
 * (may be NULL), equal to grg_label_counts / grg_set_hash of the in-core closure. */
int grg_part_label_counts(grg_part *part, uint64_t *counts, uint64_t *hash);
/* Current partition bounds: bounds[0..num_parts] (cap entries at most). */
int grg_part_bounds(grg_part *part, uint32_t cap, uint32_t *bounds, uint32_t *num_parts);
/* Rows of partition index (0-based, in bound order) of a closed set as the
 * compressed edge stream (grg_export_csr5 conventions, rows [bounds[index],
 * bounds[index+1])): the reference's per-partition spill file of
 * storeElements_c (src/main.cpp:541-596). The image is loaded on the device. */
int grg_part_export_csr5(grg_part *part, uint32_t index, uint64_t cap, uint8_t *edges, uint32_t *degree,
                         uint64_t *num_edges);

/* Checkpoint / resume. The reference keeps no superstep state (its spill files
 * hold pools only, src/main.cpp:447-456), so an interrupted run starts over.
 * Here the whole partition set -- bounds, images with stamps, the pairs each
 * run closed, run counters -- is written to one file, and a new process
 * continues from it. */

/* Write the state to path (written to path + ".tmp", then renamed over path). */
int grg_part_save(grg_part *part, const char *path);
/* A partition set rebuilt from a file written by grg_part_save, on a context
 * with the same grammar. An open set continues on grg_part_run (with the
 * filter of the interrupted run), a closed one answers grg_part_label_counts.
 * A file that is short, corrupt (checksum) or of another grammar or vertex
 * count fails with GRG_E_IO. */
int grg_part_restore(grg_part **part, grg_ctx *ctx, const char *path);
/* During grg_part_run, save to path after every `every_runs` device runs (0 =
 * never) and when the run budget stops it. */
int grg_part_set_checkpoint(grg_part *part, const char *path, uint32_t every_runs);
/* Stop grg_part_run with GRG_PAUSED once it has made max_runs device runs in
 * that call (0 = no budget): a time slice for a shared device, or a stop
 * between runs with nothing in flight. */
int grg_part_set_run_budget(grg_part *part, uint64_t max_runs);

/* Text formats (host). Grammar: readAndTransferRules (src/main.cpp:60-97);
 * names must hold GRG_MAX_LABELS*GRG_NAME_LEN bytes, label l at
 * names[(l-1)*GRG_NAME_LEN]; rules must hold 3*GRG_MAX_RULES ints. */
int grg_parse_grammar(const char *path, int *num_rules, int *rules, int *num_labels, char *names);
/* Graph header "numEdges\tnumVars" (src/main.cpp:106-115). */
int grg_parse_graph_header(const char *path, uint64_t *num_edges, uint32_t *num_vars);
/* Graph body (src/main.cpp:177-221), arrays of num_edges entries. Labels are
 * looked up in names (as filled by grg_parse_grammar); unknown labels fail with
 * GRG_E_LABEL, ids >= num_vars with GRG_E_RANGE. */
int grg_parse_graph(const char *path, int num_labels, const char *names, uint64_t num_edges,
                    uint32_t num_vars, uint32_t *src, uint32_t *dst, uint8_t *label);

/* ---- Batched closure of many independent graphs (continuous batching). The
 * reference closes one graph per process; these entry points close many in
 * one context: each job owns a vertex range [base, base+num_vars) of a
 * context-wide vertex space, all jobs share one union grammar (callers give
 * every grammar its own label range), and every round's kernels process the
 * delta records of all admitted jobs together. New jobs can be admitted
 * between steps while others are in flight. */

/* Open a batch: vertex space [0, max_vars), up to max_jobs job slots, the union
 * grammar (as grg_transfer_rules) and the filter shared by all jobs. Epsilon
 * rules are applied per job (see eps_mask of grg_batch_admit). */
int grg_batch_begin(grg_ctx *ctx, uint32_t max_vars, uint32_t max_jobs, int num_rules, const int *rules,
                    int num_labels, uint32_t filter);
/* Admit a job in slot `job`: its edges use job-local vertex ids [0, num_vars)
 * placed at `base`, labels of the union grammar. eps_mask bit l-1 = apply the
 * epsilon rule of label l to this job's vertices. on_device as for
 * grg_load_edges. The range must not overlap another admitted job. */
int grg_batch_admit(grg_ctx *ctx, uint32_t job, uint32_t base, uint32_t num_vars, uint64_t num_edges,
                    const uint32_t *src, const uint32_t *dst, const uint8_t *label, int on_device,
                    uint64_t eps_mask);
/* Run up to max_rounds semi-naive rounds over all admitted jobs (0 = until no
 * job has deltas). job_records[j] (max_jobs values, may be NULL) = delta
 * records job j had in the last round; 0 for an admitted job means it has
 * reached its fixpoint. *rounds_run = rounds that had work. */
int grg_batch_step(grg_ctx *ctx, uint32_t max_rounds, uint32_t *job_records, uint64_t *rounds_run);
/* Per-label edge counts of job `job` for the num_labels labels after
 * label_offset (its grammar's range in the union), and the edge-set hash over
 * job-local ids and labels (equal to grg_set_hash of the job closed alone). */
int grg_batch_result(grg_ctx *ctx, uint32_t job, uint32_t label_offset, uint32_t num_labels, uint64_t *counts,
                     uint64_t *hash);
/* Free a job's vertex range for reuse; only once its last step reported 0 records. */
int grg_batch_release(grg_ctx *ctx, uint32_t job);

/* Allocation-free closure. No counterpart in the reference.
 *
 * For callers that cannot allocate device memory while they run: a serving
 * loop whose device memory belongs to another allocator or budget, or a
 * process that must not let cudaMalloc/cudaFree synchronize the device while
 * other work is in flight. It runs the same load and closure kernels as
 * grg_load_edges + grg_closure, but all their scratch memory lives in one
 * static device array of GRG_NOALLOC_SCRATCH_BYTES (64 MiB), which every GPU
 * that loads this library holds until the process exits. No cudaMalloc,
 * cudaFree or other allocating routine is called, and no context is needed.
 *
 * Inputs: the grammar as for grg_transfer_rules, and num_edges edges as
 * DEVICE arrays d_src/d_dst/d_label over vertices [0, num_vars). Outputs:
 * d_label_counts (DEVICE, num_labels uint64 values), d_set_hash (DEVICE, one
 * uint64, may be NULL) and *rounds_out (host, may be NULL). stream may be NULL
 * (the legacy default stream); the call returns after the stream is idle.
 *
 * Limits: the tables take 28 bytes per (label, vertex) and the rest of the
 * array holds 198 bytes per element slot; graphs whose tables leave fewer
 * than 4096 slots, or with more edges than half the slots, are rejected with
 * GRG_E_RANGE before any launch. A graph whose loaded tables (at least 4
 * slots per non-empty row) do not fit, or whose closure outgrows the array,
 * returns GRG_E_NOMEM; the outputs are then left untouched and the next call
 * starts from a cleared array as usual.
 *
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture. The per-device address cache is written without
 * a lock: two threads making their first calls on one device at once both
 * store the same address, which is harmless. Every call reuses the same array
 * and clears it itself, so calls that overlap on the GPU race with each other.
 * The grammar travels with each launch, so a grg_closure of another context
 * running at the same time is not affected. */
#define GRG_NOALLOC_SCRATCH_BYTES (64ull << 20)
int grg_closure_noalloc(int device, void *stream, int num_rules, const int *rules, int num_labels,
                        uint32_t filter, uint32_t num_vars, uint64_t num_edges, const uint32_t *d_src,
                        const uint32_t *d_dst, const uint8_t *d_label, uint64_t *d_label_counts,
                        uint64_t *d_set_hash, uint64_t *rounds_out);

#ifdef __cplusplus
}
#endif

#endif /* GRG_H */
