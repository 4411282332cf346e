/*
 * motex_gpu.h -- C ABI of the GB300 word-based motif-extraction engine.
 *
 * This boundary replaces, in the reference MoTeX:
 *   - the all-pairs driver loop over (i, j) sequence pairs
 *     (motex.cc:494-583, including the short-sequence skip at motex.cc:536),
 *   - the per-pair extraction wrappers
 *       unsigned motifs_extraction_hd/_ed(p, m, t, n, sw, u, v)
 *       unsigned structured_motifs_extraction_hd/_ed(p, m, t, n, sw, u, v)
 *     (motexdefs.h:107-110, functions.cc:526-559, 564-705, 734-768, 773-915),
 *   - the libFLASM calls below them (flasm_hd / flasm_ed, libflasm.h),
 *   - and the quorum filter plus first-occurrence word deduplication of the
 *     writers (functions.cc:1101-1127 plain, 1166-1245 structured).
 * What stays on the host: CLI parsing, FASTA/boxes reading, header/footer
 * formatting and printing of the motif lines.
 *
 * Conventions: every entry point returns MOTEX_OK (0) or a negative
 * MOTEX_E* code and never exits the process; motex_gpu_strerror() names the
 * code and motex_gpu_last_error() gives a message for the calling thread's
 * last failure.  Host buffers are owned by the caller; device memory is
 * owned by the context.  A context is bound to one CUDA device and is not
 * thread-safe: use one context per host thread (the reference calls the
 * extraction from several OpenMP threads, each on a distinct i).
 */
#ifndef MOTEX_GPU_H
#define MOTEX_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MOTEX_OK              0
#define MOTEX_EINVAL         -1   /* bad argument (null pointer, e >= l, d not 0/1, ...) */
#define MOTEX_ENOMEM         -2   /* device or pinned host allocation failed */
#define MOTEX_ECUDA          -3   /* a CUDA runtime call failed */
#define MOTEX_EUNSUPPORTED   -4   /* size outside what the kernels implement */
#define MOTEX_ETIMEOUT       -5   /* a bounded device wait gave up (no GPU hang) */
#define MOTEX_EBUSY          -6   /* serving queue full / admission refused */
#define MOTEX_ENOTFOUND      -7   /* unknown request id */

/* Distance model, the reference's -d switch (motex.cc:126-133). */
#define MOTEX_HAMMING         0
#define MOTEX_EDIT            1

/* Longest factor length (-k, and each box length) the kernels accept. */
#define MOTEX_MAX_FACTOR    256

/*
 * Extraction parameters: the TSwitch fields the hot path reads
 * (motexdefs.h:32-61).  q, Q in percent; n, N occurrence bounds.
 * nb_gaps = 0 selects single motifs; nb_gaps > 0 selects structured motifs
 * with box 0 = (l, e) and box g+1 = (blens[g], berrs[g]) after a gap of
 * gap_min[g]..gap_max[g] symbols (the boxes file, motex.cc:302-363).
 */
typedef struct motex_params
{
    uint32_t d;
    uint32_t l;
    uint32_t e;
    uint32_t q;
    uint32_t Q;
    uint32_t n;
    uint32_t N;
    uint32_t nb_gaps;
    const uint32_t * gap_min;
    const uint32_t * gap_max;
    const uint32_t * blens;
    const uint32_t * berrs;
} motex_params;

/*
 * One reported motif, i.e. one output line of the reference writer:
 * the word (or structured word) that ends box 0 at position pos of
 * sequence seq, under gap structure strct (0 for single motifs; the index
 * into the lexicographic gap product of motex.cc:439-486 otherwise).
 * u = number of sequences holding an occurrence, v = number of occurrences.
 */
typedef struct motex_motif
{
    uint32_t seq;
    uint32_t pos;
    uint32_t strct;
    uint32_t u;
    uint32_t v;
} motex_motif;

/*
 * Result of one extraction.  motifs is in the reference's print order
 * (sequence, then end position, then structure) and already deduplicated
 * and filtered.  Free with motex_result_free().
 */
typedef struct motex_result
{
    motex_motif * motifs;
    uint32_t      count;
    uint32_t      num_seqs;
    uint64_t      ref_cells;     /* DP cells the reference computes: sum over
                                    non-skipped ordered pairs of m_i*n_j, times
                                    the number of boxes */
    uint64_t      exec_cells;    /* DP cells the GPU executed */
    uint32_t      unique_words;  /* distinct factors searched */
    uint32_t      launches;      /* kernels launched for this extraction */
    double        device_ms;     /* device time of the extraction pipeline on
                                    the resident input, CUDA events */
    double        dp_ms;         /* device time of the factor-search DP kernel
                                    alone, CUDA events on its stream */
} motex_result;

typedef struct motex_ctx motex_ctx;

/* Create / destroy a context on CUDA device `device`. */
int motex_ctx_create ( motex_ctx ** ctx, int device );
int motex_ctx_destroy ( motex_ctx * ctx );

/*
 * Whole-set extraction: all ordered pairs (i, j) of the nseq sequences,
 * i == j included, with the reference's short-sequence skip, quorum filter
 * and first-occurrence deduplication.  seqs[i] points to lens[i] bytes
 * (the FASTA symbols, upper case; no terminator needed).  Replaces
 * motex.cc:494-583 plus write_motifs' filter/dedup (functions.cc:1101-1127)
 * and write_structured_motifs' (functions.cc:1166-1245).
 */
int motex_gpu_run ( motex_ctx * ctx, const motex_params * prm,
                    const char * const * seqs, const uint32_t * lens, uint32_t nseq,
                    motex_result * out );

void motex_result_free ( motex_result * res );

/*
 * Device-resident form of motex_gpu_run, for callers that keep the input on
 * the GPU across extractions: motex_gpu_load() uploads and packs the
 * sequences once; motex_gpu_execute() runs the extraction on the resident
 * input and leaves the result on the device; motex_gpu_fetch() copies it
 * back.  load + execute + fetch == run.  From the second execute of the same
 * loaded input on, the whole device sequence is replayed as one CUDA graph.
 */
int motex_gpu_load ( motex_ctx * ctx, const motex_params * prm,
                     const char * const * seqs, const uint32_t * lens, uint32_t nseq );
int motex_gpu_execute ( motex_ctx * ctx );
int motex_gpu_fetch ( motex_ctx * ctx, motex_result * out );

/*
 * Batched, uneven-size extraction: njobs independent whole-set extractions
 * (each like motex_gpu_run, with its own sequences and parameters) walk the
 * pipeline together; the factor-search DP of all single-motif jobs that share
 * a kernel class runs as one persistent launch fed from a device work queue
 * of (job, factor tile, text chunk) items, largest first.  results[i]
 * receives job i's result (free each with motex_result_free); its dp_ms is
 * the device time of the batch's shared DP launches.
 */
typedef struct motex_job
{
    const motex_params * prm;
    const char * const * seqs;
    const uint32_t *     lens;
    uint32_t             nseq;
} motex_job;

int motex_gpu_run_batch ( motex_ctx * ctx, const motex_job * jobs, uint32_t njobs, motex_result * results );

/*
 * Serving: continuous batching of extraction requests (no counterpart in
 * the reference, which extracts one input per process run).
 *   motex_srv_create   starts `workers` worker threads on `device`, each
 *                      with its own engine context and stream, so batches
 *                      overlap on the GPU; hbm_budget_bytes bounds the
 *                      estimated device working set of the requests in
 *                      flight (0 = half of the free device memory);
 *                      max_batch bounds requests per batch; max_queue bounds
 *                      waiting requests (0 = unbounded).
 *   motex_srv_submit   copies the request and queues it; MOTEX_ENOMEM if it
 *                      can never fit the budget, MOTEX_EBUSY if the queue is
 *                      full or the server is stopping.
 *   motex_srv_wait     waits on the host up to timeout_ms (< 0: no limit)
 *                      for request `id`; returns the request's own status,
 *                      MOTEX_ETIMEOUT if it is still pending (it stays
 *                      waitable), MOTEX_ENOTFOUND for unknown or collected
 *                      ids.  The result's motif array belongs to the caller.
 *   motex_srv_destroy  finishes the queued requests, then stops.
 */
typedef struct motex_server motex_server;

typedef struct motex_srv_timing
{
    double   queue_ms;      /* submission -> batch admission */
    double   run_ms;        /* batch admission -> results ready */
    double   latency_ms;    /* submission -> results ready */
    uint32_t batch_size;    /* requests in the batch that served it */
} motex_srv_timing;

typedef struct motex_srv_stats
{
    uint64_t submitted;
    uint64_t completed;
    uint64_t failed;
    uint64_t batches;
    uint64_t cells;         /* reference DP cells of completed requests */
    uint32_t max_batch_seen;
    uint32_t queued;
    uint64_t in_use_bytes;
    uint64_t budget_bytes;
} motex_srv_stats;

int motex_srv_create ( motex_server ** srv, int device, uint64_t hbm_budget_bytes, uint32_t max_batch,
                       uint32_t workers, uint32_t max_queue );
int motex_srv_submit ( motex_server * srv, const motex_job * job, uint64_t * id );
int motex_srv_wait ( motex_server * srv, uint64_t id, int timeout_ms, motex_result * out, motex_srv_timing * timing );
int motex_srv_stats_get ( motex_server * srv, motex_srv_stats * out );
int motex_srv_destroy ( motex_server * srv );

/*
 * Plain per-pair drop-in for
 *   motifs_extraction_hd/_ed(p, m, t, n, sw, u, v)            (nb_gaps == 0)
 *   structured_motifs_extraction_hd/_ed(p, m, t, n, sw, u, v) (nb_gaps > 0)
 * (functions.cc:526-559, 734-768, 564-705, 773-915): searches every factor
 * of the pattern sequence p (length m) in the text sequence t (length n)
 * and ACCUMULATES into the caller's arrays: for factor end j and structure
 * k, u[k*m + j] += 1 if it occurs in t at all, v[k*m + j] += occurrences.
 * u and v hold m * nb_structs entries.  One extraction per call (one GPU
 * job per launch sequence): the caller's loop over pairs stays as it is.
 * Unlike the reference, this returns MOTEX_OK (0) on success.
 */
int motex_gpu_extract_pair ( motex_ctx * ctx, const motex_params * prm,
                             const char * p, uint32_t m, const char * t, uint32_t n,
                             uint32_t * u, uint32_t * v );

/*
 * Word search: the counting loop of the reference's -I mode
 * (motex.cc:938-1000, which calls motifs_extraction_hd/_ed with each motif
 * read from the -I file as the pattern and every input sequence as the
 * text; write_motifs_fore, functions.cc:2750-2829, then reads the entry of
 * the motif's last factor).  For word i, u[i] = the number of sequences
 * holding its last l symbols within e errors (distance d) at least once,
 * v[i] = the number of such occurrences over all sequences.  Sequences
 * shorter than l are skipped (motex.cc:977-982).  Words shorter than l get
 * u = v = 0.  u and v are overwritten (nwords entries each).  Plain motifs
 * only (nb_gaps = 0): the reference refuses -I with -s.  One GPU job: all
 * words against all sequences in one DP launch sequence.
 */
int motex_gpu_search ( motex_ctx * ctx, const motex_params * prm,
                       const char * const * words, const uint32_t * wlens, uint32_t nwords,
                       const char * const * seqs, const uint32_t * lens, uint32_t nseq,
                       uint32_t * u, uint32_t * v );

/* Error reporting. */
const char * motex_gpu_strerror ( int code );
const char * motex_gpu_last_error ( void );

/* Number of kernel launches issued by this context since creation. */
uint64_t motex_ctx_launches ( const motex_ctx * ctx );

/*
 * Autotuner query (no counterpart in the reference): the DP launch shape the
 * autotuner holds for the key (bit planes B, factor length l, errors e,
 * distance d) -- register words per thread W, factors per register NL,
 * block unroll UR -- from tuning done in this process or read from the file
 * MOTEX_TUNE_CACHE names (one "B l e d W NL UR F" line per entry, F the
 * Hamming form and 0 when absent; lines naming a shape the kernels do not
 * implement are ignored).  A negative NL reports the popc-free Hamming form:
 * -NL factors per register in guarded lanes.  MOTEX_ENOTFOUND if the key has
 * no entry.  Host-only: needs no GPU.
 */
int motex_tune_lookup ( int B, uint32_t l, uint32_t e, uint32_t d, int * W, int * NL, int * UR );

/*
 * Measurement utility (no counterpart in the reference): sustained
 * throughput of the integer pipes on device `device`, in 10^12 operations
 * per second, from dependent-chain microkernels with enough independent
 * chains per thread to hide latency.  lop3_tops: 3-input logic ops;
 * iadd_tops: 32-bit adds; popc_tops: population counts.
 */
int motex_probe_int_peak ( int device, double * lop3_tops, double * iadd_tops, double * popc_tops );

/*
 * Per-pair factor search that allocates nothing (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc -- code inside another
 * framework's memory pool or allocator hooks, code holding a fixed memory
 * budget, plug-ins that are only handed device buffers.  Same result as
 * motex_gpu_extract_pair for plain motifs: for every factor of p ending at
 * j, d_u[j] += 1 if it occurs in t, d_v[j] += its occurrences.  Differences:
 *   - d_p (m bytes), d_t (n bytes), d_u and d_v (m entries each) are DEVICE
 *     pointers owned by the caller; work is queued on `stream` (a
 *     cudaStream_t; 0 = default stream) of the current device, and the call
 *     returns after that stream has finished it;
 *   - symbols are coded by their index in `alphabet` (e.g. "ACGTN"; at most
 *     32 symbols); a byte outside it makes the call return MOTEX_EINVAL and
 *     leaves d_u / d_v untouched;
 *   - limits: l <= 32, m <= 32768, n <= 1048576, no structured motifs;
 *     larger sizes return MOTEX_EUNSUPPORTED.
 * All intermediate data lives in one 4 MiB static device array that every
 * GPU loading this library keeps until the process exits.  The first call
 * on a device looks up that array's address (with the device current) and
 * keeps it for the CUDA context it was looked up in; a call in a new context
 * of the device (e.g. after cudaDeviceReset) looks it up again.  Make the
 * first call on a device before any stream capture.  The call returns only
 * after `stream` has finished its work (it reads an error word back).  A
 * CUDA error already pending on the calling thread makes the call return
 * MOTEX_ECUDA at once and is left pending.  Calls share the array: calls
 * that overlap on the GPU race and must be serialised by the caller.
 */
int motex_gpu_extract_pair_static ( const motex_params * prm, const char * alphabet,
                                    const char * d_p, uint32_t m, const char * d_t, uint32_t n,
                                    uint32_t * d_u, uint32_t * d_v, void * stream );

#ifdef __cplusplus
}
#endif

#endif
