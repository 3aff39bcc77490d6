/*
 * hammingdist_gb300.h — C ABI of the GB300 (sm_103a) implementation of
 * hammingdist's pairwise Hamming-distance path (libhd).
 *
 * Plain C types only: host/device pointers, sizes and status codes. No C++
 * exception crosses this boundary; every entry point returns HD_OK (0) or a
 * negative HD_ERR_* code, and hd_last_error() holds the message (the exact
 * message text of the reference where it has one).
 *
 * Each declaration names the reference interface (ssciwr/hammingdist 1.4.0,
 * file:line) that it replaces. The reference's pybind11 module
 * (python/hammingdist.cc) is mirrored on top of this ABI by
 * hammingdist_gb300/csrc/hd_module.cpp.
 *
 * Every computation runs on the GPU. There is no CPU fallback: without a
 * usable CUDA device the calls fail with HD_ERR_NO_DEVICE.
 */
#ifndef HAMMINGDIST_GB300_H
#define HAMMINGDIST_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define HD_OK 0
#define HD_ERR_EMPTY -1          /* "Error: Empty sequence" */
#define HD_ERR_LENGTH -2         /* "Error: Sequences do not all have the same length" */
#define HD_ERR_CUDA -3           /* CUDA runtime error; message = cudaGetErrorString */
#define HD_ERR_ARG -4            /* invalid argument */
#define HD_ERR_IO -5             /* "Error: Failed to open file '<f>'" and write errors */
#define HD_ERR_INCLUDE_X_GPU -6  /* "use_gpu=True cannot be used if include_x=True, ..." */
#define HD_ERR_TIMEOUT -7        /* a bounded device-side wait ran out */
#define HD_ERR_NO_DEVICE -8      /* no usable CUDA device */
#define HD_ERR_REF_LENGTH -9     /* a record is longer than the reference sequence */
#define HD_ERR_OOM -10           /* device or pinned host allocation failed */
#define HD_ERR_STATE -11         /* object in the wrong state (e.g. released) */
#define HD_ERR_PARSE -12         /* a field std::stoi rejects (see hd_read_*) */

/* Output buffers of hd_pairwise_lt_files and the hd_read_* readers: called
 * once per output, possibly from a library thread, when its size is known
 * (hd_pairwise_lt_files: file `index`, its unique row count and
 * n_rows(n_rows-1)/2 entries; the readers: index 0, nsamples and the number
 * of values); returns the host buffer for `entries` values of the output's
 * dtype. It need not be touched yet. NULL with entries > 0 fails the call
 * with HD_ERR_ARG. Calls for different indices may run concurrently. */
typedef void *(*hd_output_fn)(void *user, uint64_t index, uint64_t n_rows, uint64_t entries);
/* hd_pairwise_lt_fasta_file asks once more, after index 0, with this index:
 * a non-NULL buffer of the same size receives a second copy of the result,
 * written while the distances run (a binding can hand it out as the first of
 * the fresh copies the reference's lt_array returns,
 * python/hammingdist.cc:47-49,65-67). NULL: no second copy. */
#define HD_OUTPUT_MIRROR UINT64_MAX

/* ---- semantics of a pairwise matrix ------------------------------------- */
/* HD_SEM_GPU: the reference's use_gpu=True semantics — the dense AND rule of
 *   src/distance_cuda.cu:57-65 on the 4-bit codes of src/hamming_impl.cc:31-44;
 *   include_x is rejected (include/hamming/hamming_impl.hh:99-102).
 * HD_SEM_CPU: the reference's use_gpu=False semantics — include_x or a
 *   consensus difference fraction below 0.005 selects the sparse rule
 *   (include/hamming/hamming_impl.hh:104-118, src/hamming_impl.cc:93-129),
 *   else the dense AND rule. Computed on the GPU all the same.            */
#define HD_SEM_GPU 0
#define HD_SEM_CPU 1

/* Rule actually used by an alignment (hd_alignment_info). */
#define HD_RULE_AND 0       /* dense AND rule, 4 bit-planes */
#define HD_RULE_SPARSE 1    /* sparse rule, X invalid (5 planes) */
#define HD_RULE_SPARSE_X 2  /* sparse rule, X a fifth symbol (6 planes) */

typedef struct hd_ctx hd_ctx;             /* one per device: streams, pools, status */
typedef struct hd_alignment hd_alignment; /* packed alignment resident in HBM */

/* Replaces distance_cuda_have_device (src/distance_cuda.cu:232-238) and
 * cuda_gpu_available (include/hamming/hamming_impl.hh:23-29): 1 if a CUDA
 * device is usable, else 0. */
int hd_device_available(void);

/* Context on `device` (ordinal). New; the reference has none (it uses the
 * default stream and cudaMalloc per call). */
int hd_ctx_create(int device, hd_ctx **out);
void hd_ctx_destroy(hd_ctx *ctx);
const char *hd_last_error(const hd_ctx *ctx);
/* Number of kernels this context has launched so far (evidence for tests and
 * benchmarks that the device path ran). */
uint64_t hd_ctx_kernel_launches(const hd_ctx *ctx);
/* Pinned host memory, reused for FASTA bytes and results. */
int hd_host_alloc(hd_ctx *ctx, size_t bytes, void **out);
void hd_host_free(hd_ctx *ctx, void *p);
/* Frees a host array returned by hd_reference_distances /
 * hd_fasta_sequence_indices. */
void hd_free(void *p);
/* Waits for all work on the context's streams. */
int hd_ctx_synchronize(hd_ctx *ctx);
/* The cudaStream_t (as void*) the context launches its kernels on, so a
 * caller can time them with CUDA events on that stream. */
void *hd_ctx_stream(const hd_ctx *ctx);

/* ---- ingest ------------------------------------------------------------- */
/* Replaces read_fasta + validate_data + to_dense_data
 * (src/hamming_impl.cc:200-242, :80-91, :190-198, :244-267) and, with
 * HD_SEM_CPU, the consensus/heuristic of include/hamming/hamming_impl.hh:
 * 95-118. `fasta` holds the raw FASTA bytes, in host memory
 * (fasta_on_device = 0; pinned memory from hd_host_alloc is fastest) or
 * device memory (1). The bytes are parsed, deduplicated (remove_duplicates:
 * unique rows in first-occurrence order) and packed into bit planes on the
 * GPU. n_limit = 0 reads every record. Errors: HD_ERR_EMPTY, HD_ERR_LENGTH,
 * HD_ERR_INCLUDE_X_GPU (semantics HD_SEM_GPU with include_x). */
int hd_alignment_from_fasta(hd_ctx *ctx, const char *fasta, uint64_t nbytes,
                            int fasta_on_device, int remove_duplicates,
                            uint64_t n_limit, int include_x, int semantics,
                            hd_alignment **out);
/* The same from a FASTA file (read_fasta's own input, src/hamming_impl.cc:
 * 200-242). Up to 16 threads pread 8 MB parts into pinned staging, and each
 * part is copied to the device as soon as it is read, so the upload runs
 * under the read. The context remembers which file its device input buffer
 * holds (path, size, inode, device, mtime, ctime): the file calls below on
 * the same unchanged file reuse those device bytes without reading or
 * copying them again. A call with FASTA bytes replaces the buffer. An
 * unreadable path fails with HD_ERR_IO, "Error: Failed to open file '<f>'". */
int hd_alignment_from_fasta_file(hd_ctx *ctx, const char *path, int remove_duplicates,
                                 uint64_t n_limit, int include_x, int semantics,
                                 hd_alignment **out);
/* from_fasta(use_gpu=True) of a FASTA file as one call
 * (include/hamming/hamming.hh:169-177 with the dense AND rule): the lower
 * triangle (dtype_bytes, max_distance as in hd_pairwise_lt) is copied to the
 * buffer out_fn returns (index 0, n_rows, entries), and *aln_out receives the
 * alignment (sequence indices; free it with hd_alignment_free). out_fn is
 * then asked for HD_OUTPUT_MIRROR (see there). For a file of 64 MB or more
 * the distances overlap the read: the file is ingested in parts that end at
 * record headers (by default after ~35% and ~65% of its bytes;
 * HAMMINGDIST_STREAM_SPLITS sets up to three splits); after each part the
 * unique rows so far (the first rows of the final result) are packed and the
 * tile rows that are complete run while the rest is read, and finished
 * ranges of the result are copied while later ones compute. Multi-line
 * records, or a file already on the device, take the plain order: read,
 * ingest, distances. Results and errors are those of
 * hd_alignment_from_fasta_file + hd_pairwise_lt. */
int hd_pairwise_lt_fasta_file(hd_ctx *ctx, const char *path, int remove_duplicates,
                              int dtype_bytes, int64_t max_distance, hd_output_fn out_fn,
                              void *user, hd_alignment **aln_out);
/* Same from n sequences held back to back in `bytes` with offsets[0..n]
 * (host memory). Replaces the DataSet(std::vector<std::string>&) path of
 * from_stringlist (src/hamming.cc:16-21). */
int hd_alignment_from_sequences(hd_ctx *ctx, const char *bytes,
                                const uint64_t *offsets, uint64_t n,
                                int include_x, int semantics,
                                hd_alignment **out);
/* Rows (after dedupe), sites per row, records read, rule in use. */
int hd_alignment_info(const hd_alignment *aln, uint64_t *n_rows,
                      uint64_t *length, uint64_t *n_input, int *rule);
/* sequence_indices of read_fasta (src/hamming_impl.cc:228): n_input entries,
 * the unique row of each input record; identity without dedupe. */
int hd_alignment_sequence_indices(const hd_alignment *aln, uint64_t *out);
void hd_alignment_free(hd_alignment *aln);

/* ---- pairwise lower triangle ------------------------------------------- */
/* Replaces distances_cuda_8bit / distances_cuda_16bit
 * (src/distance_cuda.cu:204-214; header include/hamming/distance_cuda.hh:
 * 19-25) and the dense/sparse CPU loops of include/hamming/hamming_impl.hh:
 * 120-175. Writes lt[i(i-1)/2 + j] = min(count(i, j), max_dist) for i > j,
 * n_rows(n_rows-1)/2 entries of dtype_bytes (1 = uint8, 2 = uint16,
 * 4 = uint32). max_distance is clamped like safe_int_cast
 * (include/hamming/hamming_impl.hh:37-45): above the dtype maximum it
 * saturates, negative values wrap. `out` is host memory (out_on_device = 0)
 * or device memory (1). A host output of 16 MB or more need not have been
 * touched: its pages are first written (zeros) on up to 16 threads while
 * the kernel runs, then the results are copied in. */
int hd_pairwise_lt(hd_ctx *ctx, const hd_alignment *aln, int dtype_bytes,
                   int64_t max_distance, void *out, int out_on_device);

/* Replaces distances_cuda_to_lower_triangular (src/distance_cuda.cu:
 * 216-223) with the streamed writer of partial_write_lower_triangular
 * (include/hamming/hamming_utils.hh:64-104): uint16 distances, the text is
 * formatted on the GPU and written to `path` while later rows compute.
 * With fewer than 2 rows the file is left untouched, as in the reference. */
int hd_pairwise_lt_to_file(hd_ctx *ctx, const hd_alignment *aln,
                           int64_t max_distance, const char *path);

/* ---- writers over a lower triangle held by the caller ------------------- */
/* Replaces write_lower_triangular (include/hamming/hamming_utils.hh:106-110)
 * as used by DataSet::dump_lower_triangular (include/hamming/hamming.hh:
 * 75-77). `lt` is host memory with nsamples(nsamples-1)/2 entries. */
/* ---- result files ------------------------------------------------------- */
/* Replaces DataSet::dump (include/hamming/hamming.hh:63-73): the full
 * nsamples x nsamples matrix as text, entries of row i separated by ", ",
 * one line per row, 0 on the diagonal and the matrix symmetric, read from
 * the `entries` lower-triangle values lt[i(i-1)/2 + j] (host memory; an
 * index past `entries` reads as 0). Formatted on the device, written to the
 * file in chunks while the next chunk formats. Output of the device
 * formatter is byte-identical to the reference's ofstream output. */
int hd_write_full_matrix(hd_ctx *ctx, const void *lt, uint64_t entries, uint64_t nsamples,
                         int dtype_bytes, const char *path);
/* Replaces from_lower_triangular<T> (include/hamming/hamming.hh:152-166;
 * dtype_bytes 1 = uint8_t, 2 = uint16_t): every comma-separated field of
 * every line of the file, parsed on the device with std::stoi's rules and
 * stored through safe_int_cast<T> (include/hamming/hamming_impl.hh:37-45).
 * out_fn (see hd_output_fn; index 0) receives *nsamples, inferred as the
 * reference does ((round(sqrt(8 entries + 1)) + 1) / 2), and the number of
 * values, and returns the host buffer they are copied to. A field std::stoi
 * rejects fails the call with HD_ERR_PARSE before out_fn is called, and
 * *parse_error says which exception the reference raises there: 1 =
 * std::invalid_argument (no digits), 2 = std::out_of_range (outside int).
 * An unreadable path fails with HD_ERR_IO. */
int hd_read_lower_triangular(hd_ctx *ctx, const char *path, int dtype_bytes, hd_output_fn out_fn,
                             void *user, uint64_t *entries, uint64_t *nsamples, int *parse_error);
/* Replaces from_csv / DataSet(filename) (include/hamming/hamming.hh:34-55,
 * src/hamming.cc:23-25): nsamples = number of '\n' in the file; the result
 * has nsamples(nsamples+1)/2 uint8 values, zero-initialised; line i gives
 * its first i comma-separated fields to value i(i-1)/2 + j (a line with
 * fewer repeats its last field, as std::getline leaves it in place), each
 * through std::stoi truncated to uint8. Errors and out_fn as in
 * hd_read_lower_triangular. */
int hd_read_csv(hd_ctx *ctx, const char *path, hd_output_fn out_fn, void *user, uint64_t *entries,
                uint64_t *nsamples, int *parse_error);
int hd_write_lower_triangular(hd_ctx *ctx, const void *lt, uint64_t nsamples,
                              int dtype_bytes, const char *path);
/* Replaces DataSet::dump_sparse (include/hamming/hamming.hh:79-114): lines
 * "i j d\n" for i > j and d <= threshold, in ascending row order (one of the
 * orders the reference's OpenMP build can produce). *n_lines gets the count
 * (may be NULL). */
int hd_write_sparse(hd_ctx *ctx, const void *lt, uint64_t nsamples,
                    int dtype_bytes, int64_t threshold, const char *path,
                    uint64_t *n_lines);

/* Lower-triangular text of a lower triangle already in device memory, into a
 * caller-provided device buffer, WITHOUT ANY DEVICE ALLOCATION. No
 * counterpart in the reference. For callers that cannot allocate device
 * memory: applications whose device memory is owned by their own allocator
 * or held to a fixed budget, and loops that cannot pay for cudaMalloc /
 * cudaFree (cudaFree synchronises the device). Same bytes as
 * hd_write_lower_triangular writes to a file.
 *  - Limit: nsamples <= 262144; larger inputs fail with HD_ERR_ARG before
 *    any work. The scratch is a fixed ~4.2 MB device array in the library,
 *    held on every GPU that loads it until the process exits.
 *  - The first call on a device looks up that array's device address (once
 *    per device).
 *  - *text_bytes receives the text size; if it exceeds text_capacity the
 *    call fails with HD_ERR_ARG and writes no text.
 *  - All calls share the one scratch array: calls that overlap on the GPU
 *    (other threads, other contexts on the same device) race and must not
 *    be issued. */
int hd_lower_triangular_text_noalloc(hd_ctx *ctx, const void *d_lt,
                                     uint64_t nsamples, int dtype_bytes,
                                     char *d_text, uint64_t text_capacity,
                                     uint64_t *text_bytes);

/* ---- reference distances / indices / single pair ------------------------ */
/* Replaces fasta_reference_distances (src/hamming.cc:104-141): one uint32
 * distance per FASTA record against `ref` under the rule of src/hamming.cc:
 * 128-136. *out is allocated here (free with hd_free), *n_out entries.
 * A record longer than `ref` fails with HD_ERR_REF_LENGTH (the reference
 * reads past its buffer there). */
int hd_reference_distances(hd_ctx *ctx, const char *ref, uint64_t ref_len,
                           const char *fasta, uint64_t nbytes, int include_x,
                           uint32_t **out, uint64_t *n_out);
/* The same from a FASTA file, read as in hd_alignment_from_fasta_file
 * (reusing the device bytes of the same unchanged file). After
 * hd_pairwise_lt_fasta_file on the same unchanged file, with include_x = 0
 * and `ref` as long as the records, the distances come from the packed rows
 * that call left (the rule then equals the dense AND rule), not from the
 * records' bytes; the results are the same. */
int hd_reference_distances_file(hd_ctx *ctx, const char *ref, uint64_t ref_len,
                                const char *path, int include_x, uint32_t **out,
                                uint64_t *n_out);
/* Same against a resident alignment: one distance per INPUT record (rows
 * expanded through the sequence indices). ref_len must equal the alignment's
 * length. Used by the serving loop. */
int hd_alignment_reference_distances(hd_ctx *ctx, const hd_alignment *aln,
                                     const char *ref, uint64_t ref_len,
                                     int include_x, uint32_t *out);
/* Replaces fasta_sequence_indices (src/hamming.cc:76-102). *out allocated
 * here (free with hd_free), *n_out entries. */
int hd_fasta_sequence_indices(hd_ctx *ctx, const char *fasta, uint64_t nbytes,
                              uint64_t n_limit, uint64_t **out,
                              uint64_t *n_out);
/* The same from a FASTA file, read as in hd_alignment_from_fasta_file. */
int hd_fasta_sequence_indices_file(hd_ctx *ctx, const char *path, uint64_t n_limit,
                                   uint64_t **out, uint64_t *n_out);
/* Replaces distance (src/hamming.cc:54-74) and distance_cuda
 * (src/distance_cuda.cu:225-230): one pair under the reference-distance rule.
 * Unequal lengths fail with HD_ERR_LENGTH. */
int hd_distance(hd_ctx *ctx, const char *s0, uint64_t l0, const char *s1,
                uint64_t l1, int include_x, uint32_t *out);

/* ---- batches of independent matrices ------------------------------------ */
/* No reference counterpart: the reference computes one matrix per call. A
 * batch holds jobs (alignment, dtype, max_distance, output); hd_batch_run
 * computes all of them with one persistent kernel per kernel configuration,
 * whose CTAs draw triangle tiles of every job from a device counter, biggest
 * jobs first. The launches are captured in a CUDA graph on the first run and
 * replayed on later runs of the same batch. Outputs in host memory are
 * staged on the device and copied back after the graph. */
typedef struct hd_batch hd_batch;
int hd_batch_create(hd_ctx *ctx, hd_batch **out);
int hd_batch_add(hd_batch *b, const hd_alignment *aln, int dtype_bytes,
                 int64_t max_distance, void *out, int out_on_device);
int hd_batch_run(hd_batch *b);
/* Device time of the last hd_batch_run (graph launch + copies, ms), the
 * number of persistent launches in its graph and the tiles they process. */
int hd_batch_timing(const hd_batch *b, double *ms, uint64_t *launches,
                    uint64_t *tiles);
void hd_batch_free(hd_batch *b);
/* Builds `count` alignments from `count` FASTA buffers (host memory) in
 * parallel on worker contexts with their own streams; same semantics per
 * buffer as hd_alignment_from_fasta. On error nothing is returned and the
 * message names the failing input. */
int hd_alignments_from_fasta_many(hd_ctx *ctx, uint64_t count,
                                  const char *const *fasta,
                                  const uint64_t *nbytes,
                                  int remove_duplicates, uint64_t n_limit,
                                  int include_x, int semantics,
                                  hd_alignment **out);

/* Same from FASTA files: worker contexts each read the next file into their
 * own pinned buffer and ingest it at once, so reading one file overlaps the
 * device ingest of others. An unreadable file fails with HD_ERR_IO
 * ("Error: Failed to open file '<f>'"). */
int hd_alignments_from_fasta_files(hd_ctx *ctx, uint64_t count,
                                   const char *const *paths,
                                   int remove_duplicates, uint64_t n_limit,
                                   int include_x, int semantics,
                                   hd_alignment **out);

/* Many FASTA files to their lower triangles in one pipelined call (no
 * reference counterpart: the reference computes one matrix per call, as in
 * from_fasta, include/hamming/hamming.hh:169-177).
 * - Reader threads read the files into pinned memory without waiting for
 *   the GPU.
 * - Worker contexts ingest each file as soon as it is read, on their own
 *   streams.
 * - Whenever the context's stream is idle, every ingested alignment not yet
 *   computed goes into one persistent pairwise launch.
 * - A completion thread copies each finished group to its host outputs
 *   while later files are still being read.
 * dtype_bytes[i] and max_distance[i] apply to file i as in hd_pairwise_lt.
 * alns (optional, count entries) receives the alignments, e.g. for their
 * sequence indices; free them with hd_alignment_free. */
int hd_pairwise_lt_files(hd_ctx *ctx, uint64_t count, const char *const *paths,
                         int remove_duplicates, uint64_t n_limit, int include_x, int semantics,
                         const int *dtype_bytes, const int64_t *max_distance,
                         hd_output_fn out_fn, void *user, hd_alignment **alns);

/* A view of rows [row0, row0 + n_rows) of an alignment, usable wherever an
 * alignment is (pairwise, batches, serving). It borrows the base's device
 * memory: free the view before the base. No reference counterpart. */
int hd_alignment_view(const hd_alignment *base, uint64_t row0, uint64_t n_rows,
                      hd_alignment **out);

/* ---- synthetic input (benchmarks and tests) -------------------------------- */
/* Writes n seeded synthetic FASTA records of L sites into device memory
 * (d_out, capacity bytes; d_out = NULL only reports *nbytes): a root uniform
 * over ACGT, substitution probability p, N runs (about n_rate per site, 1-50
 * long), '-' runs of 0..dash_max at both ends; records ">s%09d\n" + sites +
 * "\n". Every byte is a function of (seed, record, site). No reference
 * counterpart. */
int hd_synthetic_fasta(hd_ctx *ctx, uint64_t n, uint64_t L, double p,
                       uint64_t seed, uint32_t dash_max, double n_rate,
                       void *d_out, uint64_t capacity, uint64_t *nbytes);

/* ---- serving --------------------------------------------------------------- */
/* A request loop over resident alignments with continuous batching. No
 * reference counterpart. Requests are admitted in arrival order while the
 * device output bytes they need fit in output_budget_bytes (a request larger
 * than the budget runs alone); every admitted request is folded into one
 * wave (one persistent pairwise kernel over all matrices' tiles, plus the
 * query kernels) launched on a free worker stream, with up to max_waves
 * waves on the device at once. Results stay in the server until released.
 *  - reference: distances of `query` (length = the alignment's length) to
 *    every input record, uint32 (the fasta_reference_distances rule);
 *  - pairwise: lower triangle of rows [row0, row0 + n_rows), dtype 1 or 2;
 *  - sparse: "i j d\n" text (window-relative i > j, d <= threshold < 255)
 *    in ascending rows, as DataSet::dump_sparse writes it. */
typedef struct hd_server hd_server;
int hd_server_create(hd_ctx *ctx, uint64_t output_budget_bytes, int max_waves,
                     hd_server **out);
int hd_server_add_alignment(hd_server *s, const hd_alignment *aln, uint32_t *id);
int hd_server_submit_reference(hd_server *s, uint32_t aln_id, const char *query,
                               uint64_t len, uint64_t *ticket);
int hd_server_submit_pairwise(hd_server *s, uint32_t aln_id, uint64_t row0,
                              uint64_t n_rows, int dtype_bytes,
                              int64_t max_distance, uint64_t *ticket);
int hd_server_submit_sparse(hd_server *s, uint32_t aln_id, uint64_t row0,
                            uint64_t n_rows, int64_t threshold,
                            uint64_t *ticket);
/* Waits up to timeout_s for the request; returns its status. */
int hd_server_wait(hd_server *s, uint64_t ticket, double timeout_s);
/* Result of a finished request: bytes, element/line count, latency from
 * submission to completion and the part of it spent waiting for admission. */
int hd_server_result(hd_server *s, uint64_t ticket, const void **data,
                     uint64_t *bytes, uint64_t *count, double *latency_ms,
                     double *queue_ms);
int hd_server_release(hd_server *s, uint64_t ticket);
/* Withdraws a request that is still queued (not yet admitted): it finishes
 * with HD_ERR_STATE "request cancelled". Admitted requests cannot be
 * cancelled (HD_ERR_STATE). */
int hd_server_cancel(hd_server *s, uint64_t ticket);
int hd_server_stats(hd_server *s, uint64_t *waves, uint64_t *completed,
                    uint64_t *max_inflight, uint64_t *bytes_in_use);
/* Stops admitting, fails queued requests, drains the waves on the device. */
void hd_server_free(hd_server *s);

/* ---- autotuning ------------------------------------------------------------ */
/* Times every kernel configuration of both distance engines for each
 * (n bucket <= max_n_bucket, L bucket, dtype) with the GPU filled, and keeps
 * the fastest per bucket in the context: for the bit-plane engine the tile
 * edge (64/128 = 4/8 rows per thread) and TMA staging depth (2-4), for the
 * tensor-core engine the L2 band (8, 16 or 32 tile rows) and the item shape
 * (one or two 128-row tiles). Then, per L bucket, it times single matrices
 * of growing size on both engines and keeps the launch size (single-row-tile
 * items) from which the tensor-core engine wins. Without a table (or with
 * HAMMINGDIST_TILE=<tile>x<stages>, HAMMINGDIST_MMA_BAND, HAMMINGDIST_MMA_ROWS,
 * HAMMINGDIST_MMA_MIN_ITEMS) built-in choices apply. No reference
 * counterpart (the reference has one kernel shape,
 * src/distance_cuda.cu:142-155). */
int hd_autotune(hd_ctx *ctx, uint64_t max_n_bucket);
int hd_tune_lookup(hd_ctx *ctx, uint64_t n_rows, uint64_t length,
                   int dtype_bytes, int *tile, int *stages);
/* The tensor-core engine's settings that apply to a matrix of n_rows x length
 * sites: L2 band (tile rows), row tiles per item (1 or 2) and the launch
 * size from which a launch goes to that engine. No reference counterpart. */
int hd_tune_lookup_mma(hd_ctx *ctx, uint64_t n_rows, uint64_t length,
                       int dtype_bytes, int *band, int *rows, uint64_t *min_items);
int hd_tune_save(hd_ctx *ctx, const char *path);
int hd_tune_load(hd_ctx *ctx, const char *path);

/* ---- measurement --------------------------------------------------------- */
/* Phase tracing, off by default (HAMMINGDIST_TRACE=1 in the environment
 * turns it on when a context is created). While on, hd_alignment_from_fasta,
 * hd_pairwise_lt and hd_reference_distances record a CUDA event on the
 * context's stream at each phase boundary (upload, parse, dedupe, consensus,
 * pack, pairwise, copy to host, ...) and an NVTX range per call; the
 * durations are read once when the call ends. hd_trace_last returns the text
 * of the last traced call ("<call>: <phase> <ms> ms, ..., stream time <ms>
 * ms"), valid until the next call on the context. Stands in for the
 * reference's wall-clock timing lines (include/hamming/hamming_impl.hh:74-87)
 * and its CUDA-event timers (src/distance_cuda.cu:96-99,167-178). */
int hd_trace_enable(hd_ctx *ctx, int on);
const char *hd_trace_last(const hd_ctx *ctx);
/* Integer-pipe peaks of this device, measured by timing dependent LOP3 and
 * POPC chains (lane operations per second) and the pairwise inner loop's
 * instruction mix from registers alone at 16 warps per SM (4 LOP3 + POPC +
 * IMAD per 32 pair-sites; pair-sites per second). No reference counterpart. */
int hd_measure_int_peaks(hd_ctx *ctx, double *lop3_per_s, double *popc_per_s,
                         double *mix_pair_sites_per_s);
/* Dense FP4 tensor-core rate of this device (FLOP per second): one CTA per SM
 * issues back-to-back tcgen05.mma.kind::mxf4.block_scale (E2M1, M=128,
 * N=256, K=64) on shared-memory operands, the instruction of the
 * tensor-core distance engine. No reference counterpart. */
int hd_measure_mma_peak(hd_ctx *ctx, double *fp4_flop_per_s);
/* Failure-path self-test: a kernel waits, with the bounded wait of the
 * pairwise kernel and a limit of limit_ns (<= 1 s), on an mbarrier that is
 * never completed; *status receives the kernel's status word (1 = the wait
 * ran out) and *waited_ms how long it waited. Nothing faults or hangs, and
 * the context stays usable. No reference counterpart. */
int hd_selftest_wait_timeout(hd_ctx *ctx, uint64_t limit_ns, int *status,
                             double *waited_ms);
/* Device time of the last pairwise kernel launch sequence (ms, CUDA events on
 * the launching stream) and the number of tiles it processed. */
int hd_last_pairwise_timing(const hd_ctx *ctx, double *ms, uint64_t *tiles);
/* Tensor-core work of the last hd_pairwise_lt: the multiply-adds its
 * launches performed for the lower triangle (pairs x operand values per
 * pair; 0 if the bit-plane engine computed it). No reference counterpart. */
int hd_last_pairwise_work(const hd_ctx *ctx, double *mma_macs);

#ifdef __cplusplus
}
#endif
#endif /* HAMMINGDIST_GB300_H */
