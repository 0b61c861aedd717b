/*
 * nqueens_gb300.h -- C ABI of libnqgpu.so, the GB300 (sm_103a) N-Queens
 * constellation engine.
 *
 * Plain C types only (no torch, no C++): bind it from ctypes, cgo, JNI or
 * C/C++.  Every function that can fail returns an int status: NQ_OK (0) or a
 * negative NQ_E* code; nq_last_error() gives the message of the handle's last
 * failure.  A device-side failure is always an error status, never a partial
 * count.
 *
 * Each declaration names the reference interface it replaces, by file:line in
 * suzukiiichiro/N-Queens.
 */
#ifndef NQUEENS_GB300_H
#define NQUEENS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NQ_OK 0
#define NQ_EINVAL (-1)     /* bad argument */
#define NQ_ESTACK (-2)     /* a task is deeper than the launch's stack (never a partial count) */
#define NQ_ETIMEOUT (-3)   /* a bounded wait ran out */
#define NQ_ECUDA (-4)      /* CUDA runtime error (message in nq_last_error) */
#define NQ_ENOMEM (-5)     /* device or host allocation failed */
#define NQ_EPRESET (-6)    /* preset too deep for N: the reference raises on the negative shift */
#define NQ_EBUSY (-7)      /* asynchronous work still running */

/* The reference's 16-byte task record, little-endian u32 fields, exactly the
 * layout of its constellations_N{N}_{P}.bin files
 * (14Bit_codon_GPU/356Py_savesp_narrow.py:2981-2986). */
typedef struct nq_record {
  uint32_t ld, rd, col, startijkl;
} nq_record;

typedef struct nq_handle nq_handle;

const char *nq_version(void);
const char *nq_strerror(int status);

/* One handle = one device + one CUDA stream.  Calls on a handle are
 * serialised by the caller; different handles are independent. */
int nq_create(nq_handle **out, int device);
void nq_destroy(nq_handle *h);
int nq_last_error(const nq_handle *h, char *buf, size_t cap);
/* Name of the handle's GPU (the key of the autotuner's tables). */
int nq_device_name(const nq_handle *h, char *buf, size_t cap);
/* Multiprocessor count of the handle's GPU. */
int nq_device_sms(const nq_handle *h, int *sms);

/* Launch knobs chosen by the autotuner: threads per block (64, 128 or 256),
 * grid (0 = one wave of resident blocks) and split depth (-1 = automatic,
 * 0..3 = expand every task that many levels on the device before the DFS, so
 * the queue holds many small subtasks instead of few large ones). */
int nq_set_config(nq_handle *h, int block, int grid, int split_depth);
int nq_get_config(const nq_handle *h, int *block, int *grid, int *split_depth);

/* Order of the DFS queue of single-N counts: 0 = generator order (split
 * subtasks task after task), 1 = largest estimated subtree first, sorted on
 * the device.  Replaces the reference's cost-key reorder of its task list
 * before launch (14Bit_codon_GPU/356Py_savesp_narrow.py:4310-4372, risk table
 * :3646-3748; sort modes :2445-2541).  Counts do not depend on the order. */
int nq_set_queue_order(nq_handle *h, int mode);
int nq_get_queue_order(const nq_handle *h, int *mode);

/* select_dynamic_preset_queens (356Py_savesp_narrow.py:5744-5753). */
int nq_preset_for(int N);

/* gen_constellations (356Py_savesp_narrow.py:2837-2926) on the host: writes
 * up to `cap` records and returns the total count (call with cap = 0 to size
 * the buffer), or a negative status.  5 <= N <= 27. */
int64_t nq_gen_constellations(int N, int preset, nq_record *out, int64_t cap);
/* Same records with the reference's full-width masks (Python ints there),
 * as its 40-byte solutions_*_v2.bin files store them
 * (13Bit_codon/18Py_constellations_GPU_cuda_codon.py:1841-1855). */
int64_t nq_gen_constellations_wide(int N, int preset, uint64_t *ld, uint64_t *rd, uint64_t *col,
                                   uint32_t *startijkl, int64_t cap);

/* exec_solutions(N, constellations, use_gpu=True)
 * (356Py_savesp_narrow.py:2228-2578, kernel launch :1749-1835): host records
 * in, host results out.  `solutions` (nullable) receives each record's count
 * times its symmetry weight (the reference's c["solutions"]); `total`
 * receives their sum.  6 <= N <= 27. */
int nq_exec_solutions(nq_handle *h, int N, const nq_record *records, int64_t m, uint64_t *solutions,
                      uint64_t *total);

/* Same on device-resident buffers on `stream` (NULL: the handle's stream).
 * `start_min` is the smallest start row (startijkl >> 20) over the records,
 * or -1 to use the bound 1.  d_total (device, 1 x u64) is overwritten.  The
 * call waits once for a 40-byte read-back (the subtask count and the deepest
 * schedule, which size the DFS queue and stacks) before launching the DFS,
 * then returns.  Call nq_sync() to wait for the result and collect the
 * status. */
int nq_exec_solutions_device(nq_handle *h, int N, const nq_record *d_records, int64_t m, int start_min,
                             uint64_t *d_solutions, uint64_t *d_total, void *stream);
/* Waits for the handle's last nq_exec_solutions_device call (an event
 * recorded on its stream; other handles, batches and streams are not waited
 * for) and returns its device status; with nothing outstanding, waits for the
 * handle's own stream. */
int nq_sync(nq_handle *h);
/* Device time of the last exec_solutions call's prepare and DFS kernels
 * (CUDA events recorded on the launching stream); waits for them. */
int nq_last_kernel_ms(nq_handle *h, float *prepare_ms, float *dfs_ms);
/* Split depth used by the last exec_solutions call and the length of the
 * DFS queue it built (records, or subtasks when split). */
int nq_last_run_info(const nq_handle *h, int *split_depth, int64_t *queued);

/* exec_solutions for callers that cannot allocate device memory -- no
 * counterpart in the reference.  Some callers must not call cudaMalloc or
 * cudaFree once running: a serving process whose device memory is owned by
 * another allocator or a fixed budget, or a latency-critical loop where an
 * allocation's implicit device synchronisation would stall other streams.
 * Same inputs and outputs as nq_exec_solutions_device (device records in,
 * device per-record counts (nullable) and total out, on `stream`, NULL = the
 * legacy default stream), but no handle and no allocation of any kind: the
 * scratch is one fixed __device__ array of about 15 MiB inside the library,
 * held by every GPU that loads it until exit.  Limit: m <= 131072 records and
 * schedules up to 24 depths (N - start_min <= 25); larger inputs are rejected
 * with NQ_EINVAL, never truncated.  No task splitting.  The first call on each
 * device looks the array's address up (cudaGetSymbolAddress) with that device
 * current; with lazy module loading that first call is also when the array
 * and the kernels are loaded onto the device, so make it once at start-up --
 * before another allocator reserves the GPU's memory, and before any stream
 * capture.  The address is kept for the life of the process: after a
 * cudaDeviceReset of that device the library must be reloaded.  Every call
 * shares the one array, so calls that overlap on the GPU race: serialise
 * them.  The call waits for its stream before it returns, and returns the
 * device status. */
int nq_exec_solutions_noalloc(int N, const nq_record *d_records, int64_t m, int start_min, uint64_t *d_solutions,
                              uint64_t *d_total, void *stream);

/* Autotuner: times the whole count of N (its default preset's task list,
 * resident on the device) for every threads-per-block (64/128/256) and split
 * depth (0..3), `repeats` timed runs each after one warm-up, checks that every
 * configuration gives the same total, leaves the fastest set on the handle and
 * reports it.  Replaces hand-setting the reference's launch knobs
 * (gpu_block / gpu_max_blocks of exec_solutions, 356Py_savesp_narrow.py:2228). */
int nq_tune(nq_handle *h, int N, int repeats, int *best_block, int *best_split, float *best_ms);

/* Whole-board total for N, the loop body of the reference's main()
 * (356Py_savesp_narrow.py:6036-6046): brute force on the GPU for N <= 5
 * (the reference's _bit_total, :5755-5767), the constellation path above.
 * preset <= 0 selects nq_preset_for(N).  The records are generated and
 * counted in chunks (the reference's streamed generation,
 * gen_constellations_stream_to_bin, :2988-3084), so host memory stays bounded
 * at the largest boards: the next chunk is generated while the previous one
 * counts on the GPU. */
int nq_count(nq_handle *h, int N, int preset, uint64_t *total);
/* The canonical start constellations of N (6 <= N <= 27; packed
 * i<<15 | j<<10 | k<<5 | l, ascending), the first stage of
 * gen_constellations (356Py_savesp_narrow.py:2837-2880).  Writes them when
 * out != NULL and cap is large enough; returns their number or a negative
 * status.  Host only. */
int64_t nq_start_constellations(int N, int32_t *out, int64_t cap);
/* The records that start constellations [first, first + count) of
 * nq_start_constellations' list expand into (preset <= 0: nq_preset_for(N)),
 * in the order nq_gen_constellations lists them: the per-start loop of the
 * reference's streamed task writer (gen_constellations_stream_to_bin,
 * 356Py_savesp_narrow.py:2988-3084), a range at a time.  Writes them when
 * out != NULL and cap is large enough; returns their number or a negative
 * status (a range outside the list is NQ_EINVAL).  Host only. */
int64_t nq_gen_constellations_starts(int N, int preset, int64_t first, int64_t count, nq_record *out, int64_t cap);
/* The part of nq_count(N, preset) that comes from start constellations
 * [first, first + count) of nq_start_constellations' list: the records those
 * starts expand into (preset <= 0: nq_preset_for(N)), streamed the same way.
 * Totals over a partition of the list add up to the whole-board total, so a
 * long count can be cut at start boundaries and resumed -- the reference's
 * restart unit is the chunk of its task list (chunk_only / debug_chunk_start,
 * 356Py_savesp_narrow.py:2418-2435, with a progress TSV, :3330-3338).  A range
 * outside the list is NQ_EINVAL; an empty range counts 0. */
int nq_count_starts(nq_handle *h, int N, int preset, int64_t first, int64_t count, uint64_t *total);
/* Records per chunk of nq_count (0: the default, 8 Mi records, about 32 MB of
 * host records per chunk; one chunk up to N=21). */
int nq_set_chunk_records(nq_handle *h, int64_t records);
/* Chunks and records of the handle's last nq_count. */
int nq_last_count_info(const nq_handle *h, int64_t *chunks, int64_t *records);

/* Unique (distinct under rotation and reflection) and total counts by the
 * symmetry method (11Bit_Python/07Py_bit_symmetry.py:65-200; GPU form
 * 10Bit_CUDA/01CUDA_Bit_Symmetry.cu:627-960).  4 <= N <= 27.  Runs on the
 * handle's device and stream with buffers the handle keeps between calls;
 * failures are reported through nq_last_error like every other call. */
int nq_count_unique(nq_handle *h, int N, uint64_t *unique, uint64_t *total);

/* Completions of a board with k pre-placed queens (rows[i], cols[i]; column c
 * is bit c): the number of full placements that contain them.  No reference
 * counterpart (the reference counts whole boards only); brute-force checked. */
int nq_count_completions(nq_handle *h, int N, int k, const int *rows, const int *cols, uint64_t *count);

/* Diagnostic: the root frame {ld, rd, col, avail}, info word and compact
 * per-depth schedule words that the prepare kernel derives from one record
 * (build_soa_for_range, 356Py_savesp_narrow.py:1971-2169, plus the SQ* walk
 * of :689-756), computed by the same code on the host.  Returns the number
 * of words (T+1), 0 for a task without DFS work, or a negative status. */
int nq_debug_task_schedule(int N, nq_record rec, uint32_t root[4], uint32_t *info, uint32_t *words, int cap);

/* Diagnostic: the host-built tasks of a completion query (see
 * nq_count_completions), wide format: per task root {ld, rd, col, avail},
 * info word and (T+1) word pairs {x, RA} at words + task * 2 * stride.
 * *fixed_count (nullable) receives the part of the count settled without a
 * task (1 when the pre-placed queens already fill the board, else 0).
 * Returns the task count (call with cap = 0 to size), or a negative status. */
int64_t nq_debug_completion_tasks(int N, int k, const int *rows, const int *cols, int min_tasks,
                                  uint32_t *roots, uint32_t *infos, uint32_t *words, int stride, int64_t cap,
                                  uint64_t *fixed_count);

/* Diagnostic: measured INT32 instruction throughput of the device (thread
 * instructions per second) for kind 0 = lop3, 1 = add, 2 = shf, 3 = a 1:1:1
 * mix; the denominator of the DFS kernel's integer-ALU roofline. */
int nq_int32_peak(nq_handle *h, int kind, double *ops_per_s);

/* ---- batches: many jobs in one persistent launch ---- */
#define NQ_JOB_COUNT 0        /* whole-board total of N (preset 0 = nq_preset_for) */
#define NQ_JOB_COMPLETION 1   /* completions of the k pre-placed queens */
typedef struct nq_job {
  int32_t kind, N, preset, k;
  int8_t rows[8], cols[8];
} nq_job;

typedef struct nq_batch nq_batch;

/* Builds every job's tasks, uploads them once and keeps them resident. */
int nq_batch_create(nq_handle *h, const nq_job *jobs, int njobs, nq_batch **out);
int64_t nq_batch_tasks(const nq_batch *b);
/* Grid of the batch's persistent launch (0 = one wave of resident blocks on the
 * whole GPU).  A smaller grid leaves SMs to batches running beside it. */
int nq_batch_set_grid(nq_batch *b, int grid);
/* Resident DFS blocks on the whole GPU for the handle's block size and a stack
 * of maxt frames (wide: batch schedule words). */
int nq_resident_blocks(nq_handle *h, int wide, int maxt, int *blocks);
/* Resident DFS blocks on the whole GPU for this batch's own launch (its block
 * size, schedule word and stack depth): the unit nq_batch_set_grid shares out.
 * No counterpart in the reference (it runs one N per process). */
int nq_batch_resident_blocks(const nq_batch *b, int *blocks);
/* Upper estimate of the device bytes a batch holding this one job takes
 * (records, tasks, schedules and split queue) on a GPU with `sms`
 * multiprocessors at split depth `split_depth` (-1 automatic), computed on the
 * host without a device or any allocation: admission control sizes a job
 * before building it.  No counterpart in the reference (it runs one N per
 * process).  Returns the bytes or a negative status. */
int64_t nq_job_device_bytes(const nq_job *job, int sms, int split_depth);
/* Device bytes the batch holds, and host-to-device bytes its build copied
 * (records of count jobs, tasks of completion jobs). */
int64_t nq_batch_device_bytes(const nq_batch *b);
int64_t nq_batch_h2d_bytes(const nq_batch *b);
/* All jobs in one persistent launch (use_graph: replay a captured CUDA graph). */
int nq_batch_run(nq_batch *b, int use_graph, uint64_t *totals);
/* One launch and one read-back per job (the plain form, for comparison). */
int nq_batch_run_plain(nq_batch *b, uint64_t *totals);
/* Asynchronous form on the batch's own stream, so batches overlap on the
 * device: submit, then poll (waits up to max_wait_us; NQ_EBUSY while
 * running). */
int nq_batch_submit(nq_batch *b, int use_graph);
int nq_batch_poll(nq_batch *b, uint64_t *totals, int64_t max_wait_us);
void nq_batch_destroy(nq_batch *b);

#ifdef __cplusplus
}
#endif
#endif /* NQUEENS_GB300_H */
