/*
 * szp_gb300.h -- C ABI of libszp_gb300.so, a GB300 (sm_103a) implementation
 * of SZp's float32 fastmode1 / fastmode2 codec.
 *
 * The first group of functions keeps the names, arguments, return values and
 * ownership rules of SZp's own API, so a program linked against libszp can
 * link against this library instead.  Compression and decompression run as
 * CUDA kernels on the current device; host buffers are staged through device
 * memory kept by the library.  Streams are byte-identical to the reference's
 * for the same input, error bound, block size and segment count T.
 *
 * T, the number of contiguous segments of a stream, is the reference's
 * OpenMP thread count: by default it is omp_get_max_threads() of the calling
 * process (OMP_NUM_THREADS), exactly as the reference decides it, and
 * szp_gb300_set_segments() overrides it.  A stream must be decompressed with
 * the T it was made with (the reference has the same rule).
 *
 * Errors: the reference functions keep their conventions (NULL return, or an
 * *outSize of 0 for the _arg compressors) and record a message readable with
 * szp_gb300_last_error().  Extension functions return an SZP_GB300_* status.
 */
#ifndef SZP_GB300_H
#define SZP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Constants with the reference's values (SZp/include/szp_defines.h:19-37). */
#ifndef ABS
#define ABS 0
#endif
#ifndef REL
#define REL 1
#endif
#ifndef SZP_NONRANDOMACCESS
#define SZP_NONRANDOMACCESS 1
#endif
#ifndef SZP_RANDOMACCESS
#define SZP_RANDOMACCESS 2
#endif
#ifndef SZ_FLOAT
#define SZ_FLOAT 0
#endif
#ifndef SZ_DOUBLE
#define SZ_DOUBLE 1
#endif

/* ---- reference entry points ------------------------------------------- */

/* Replaces SZp/include/szp.h:33 (SZp/src/szp.cc:23-116).  fastMode 1 or 2,
 * dataType SZ_FLOAT (eb = (float)absErrBound, or REL: (max-min)*(float)rel)
 * or SZ_DOUBLE (any other dataType, as in the reference: double data,
 * eb = absErrBound or (max-min)*rel in double, an 8-byte eb header).  Returns
 * a malloc'd stream the caller free()s; *outSize gets its length.  NULL on
 * error. */
unsigned char *szp_compress(int fastMode, int dataType, void *data, size_t *outSize, int errBoundMode,
                            double absErrBound, double relBoundRatio, size_t nbEle, int blockSize);

/* Replaces SZp/include/szp.h:36 (SZp/src/szp.cc:118-179).  bytes is a whole
 * stream (eb header first).  byteLength, ignored by the reference, bounds
 * the bytes read here; a value smaller than the stream header makes the
 * library find the length by walking the last segment on the host.  Returns
 * a malloc'd float[nbEle] (SZ_FLOAT) or double[nbEle] (any other dataType),
 * or NULL on error. */
void *szp_decompress(int fastMode, int dataType, unsigned char *bytes, size_t byteLength, size_t nbEle,
                     int blockSize);

/* Replaces SZp/include/szp_float.h:30 (SZp/src/szp_float.cc:148-309). */
unsigned char *szp_float_openmp_threadblock(float *oriData, size_t *outSize, float absErrBound, size_t nbEle,
                                            int blockSize);

/* Replaces SZp/include/szp_float.h:33 (SZp/src/szp_float.cc:314-480).  The
 * reference's callers size output as 4 + 4*nbEle bytes (SZp/src/szp.cc:53);
 * a stream that would not fit that is not written and *outSize is 0. */
void szp_float_openmp_threadblock_arg(unsigned char *output, float *oriData, size_t *outSize, float absErrBound,
                                      size_t nbEle, int blockSize);

/* Replaces SZp/include/szp_float.h:36 (SZp/src/szp_float.cc:482-605): the
 * T = 1 stream. */
void szp_float_single_thread_arg(unsigned char *output, float *oriData, size_t *outSize, float absErrBound,
                                 size_t nbEle, int blockSize);

/* Replaces SZp/include/szp_float.h:39 (SZp/src/szp_float.cc:607-750).
 * Same stream as szp_float_single_thread_arg; returns the reference's
 * `total_memaccess` tally for that stream (its own count of the bytes each
 * statement of the CPU loop touches), 0 on an error. */
size_t szp_float_single_thread_arg_record(unsigned char *output, float *oriData, size_t *outSize,
                                          float absErrBound, size_t nbEle, int blockSize);

/* Replaces SZp/include/szp_float.h:43 (SZp/src/szp_float.cc:752-912). */
unsigned char *szp_float_openmp_threadblock_randomaccess(float *oriData, size_t *outSize, float absErrBound,
                                                         size_t nbEle, int blockSize);

/* Replaces SZp/include/szp_float.h:47 (SZp/src/szp_float.cc:914-1076). */
void szp_float_openmp_threadblock_randomaccess_arg(unsigned char *output, float *oriData, size_t *outSize,
                                                   float absErrBound, size_t nbEle, int blockSize);

/* Replaces SZp/include/szpd_float.h:21 (SZp/src/szpd_float.cc:23-128).
 * cmpBytes points just past the 4-byte eb header, as in the reference. */
float *szp_float_decompress_openmp_threadblock(size_t nbEle, float absErrBound, int blockSize,
                                               unsigned char *cmpBytes);

/* Replaces SZp/include/szpd_float.h:23 (SZp/src/szpd_float.cc:320-423). */
void szp_float_decompress_openmp_threadblock_arg(float *newData, size_t nbEle, float absErrBound, int blockSize,
                                                 unsigned char *cmpBytes);

/* Replaces SZp/include/szpd_float.h:25 (SZp/src/szpd_float.cc:130-214). */
void szp_float_decompress_single_thread_arg(float *newData, size_t nbEle, float absErrBound, int blockSize,
                                            unsigned char *cmpBytes);

/* Replaces SZp/include/szpd_float.h:27 (SZp/src/szpd_float.cc:216-318);
 * returns the reference's `total_memaccess` tally, 0 on an error. */
size_t szp_float_decompress_single_thread_arg_record(float *newData, size_t nbEle, float absErrBound,
                                                     int blockSize, unsigned char *cmpBytes);

/* Replaces SZp/include/szpd_float.h:29 (SZp/src/szpd_float.cc:425-531). */
float *szp_float_decompress_openmp_threadblock_randomaccess(size_t nbEle, float absErrBound, int blockSize,
                                                            unsigned char *cmpBytes);

/* Replaces SZp/include/szpd_float.h:31 (SZp/src/szpd_float.cc:533-637). */
void szp_float_decompress_openmp_threadblock_randomaccess_arg(float *newData, size_t nbEle, float absErrBound,
                                                              int blockSize, unsigned char *cmpBytes);

/* float64 data (SZp/include/szp_double.h, szpd_double.h): the same streams
 * with an 8-byte big-endian eb, q = (int)(x * (1/eb)) with a double product
 * and x' = (double)q * eb.  The _arg compressors expect 8 + 8*nbEle bytes of
 * output; the decompressors' cmpBytes points just past the 8-byte eb. */

/* Replaces SZp/include/szp_double.h:30 (SZp/src/szp_double.cc:149-309). */
unsigned char *szp_double_openmp_threadblock(double *oriData, size_t *outSize, double absErrBound, size_t nbEle,
                                             int blockSize);

/* Replaces SZp/include/szp_double.h:33 (SZp/src/szp_double.cc:320-484). */
void szp_double_openmp_threadblock_arg(unsigned char *output, double *oriData, size_t *outSize,
                                       double absErrBound, size_t nbEle, int blockSize);

/* Replaces SZp/include/szp_double.h:36 (SZp/src/szp_double.cc:486-611): T = 1. */
void szp_double_single_thread_arg(unsigned char *output, double *oriData, size_t *outSize, double absErrBound,
                                  size_t nbEle, int blockSize);

/* Replaces SZp/include/szp_double.h:39 (SZp/src/szp_double.cc:613-757);
 * returns the reference's `total_memaccess` tally, 0 on an error. */
size_t szp_double_single_thread_arg_record(unsigned char *output, double *oriData, size_t *outSize,
                                           double absErrBound, size_t nbEle, int blockSize);

/* Replaces SZp/include/szp_double.h:43 (SZp/src/szp_double.cc:759-920). */
unsigned char *szp_double_openmp_threadblock_randomaccess(double *oriData, size_t *outSize, double absErrBound,
                                                          size_t nbEle, int blockSize);

/* Replaces SZp/include/szp_double.h:47 (SZp/src/szp_double.cc:922-1090). */
void szp_double_openmp_threadblock_randomaccess_arg(unsigned char *output, double *oriData, size_t *outSize,
                                                    double absErrBound, size_t nbEle, int blockSize);

/* Replaces SZp/include/szpd_double.h:21 (SZp/src/szpd_double.cc:23-128). */
double *szp_double_decompress_openmp_threadblock(size_t nbEle, double absErrBound, int blockSize,
                                                 unsigned char *cmpBytes);

/* Replaces SZp/include/szpd_double.h:23 (SZp/src/szpd_double.cc:323-429). */
void szp_double_decompress_openmp_threadblock_arg(double *newData, size_t nbEle, double absErrBound,
                                                  int blockSize, unsigned char *cmpBytes);

/* Replaces SZp/include/szpd_double.h:25 (SZp/src/szpd_double.cc:130-217). */
void szp_double_decompress_single_thread_arg(double *newData, size_t nbEle, double absErrBound, int blockSize,
                                             unsigned char *cmpBytes);

/* Replaces SZp/include/szpd_double.h:27 (SZp/src/szpd_double.cc:219-321);
 * returns the reference's `total_memaccess` tally, 0 on an error. */
size_t szp_double_decompress_single_thread_arg_record(double *newData, size_t nbEle, double absErrBound,
                                                      int blockSize, unsigned char *cmpBytes);

/* Replaces SZp/include/szpd_double.h:29 (SZp/src/szpd_double.cc:431-534). */
double *szp_double_decompress_openmp_threadblock_randomaccess(size_t nbEle, double absErrBound, int blockSize,
                                                              unsigned char *cmpBytes);

/* Replaces SZp/include/szpd_double.h:31 (SZp/src/szpd_double.cc:536-645). */
void szp_double_decompress_openmp_threadblock_randomaccess_arg(double *newData, size_t nbEle, double absErrBound,
                                                               int blockSize, unsigned char *cmpBytes);

/* ---- extensions (no counterpart in the reference) ---------------------- */

#define SZP_GB300_OK 0
#define SZP_GB300_EINVAL -1     /* bad argument */
#define SZP_GB300_ECUDA -2      /* CUDA runtime error */
#define SZP_GB300_ECAPACITY -3  /* output buffer too small */
#define SZP_GB300_ECORRUPT -4   /* malformed stream */
#define SZP_GB300_ETIMEOUT -5   /* a device-side wait gave up */
#define SZP_GB300_ENOMEM -6     /* allocation failed */

/* Segment count T for the calls of this process; 0 restores the default
 * (omp_get_max_threads()). */
void szp_gb300_set_segments(int segments);
int szp_gb300_get_segments(void);

/* Message and status of the calling thread's last failed call. */
const char *szp_gb300_last_error(void);
int szp_gb300_last_status(void);

/* Largest stream for nbEle floats (header included). */
size_t szp_gb300_max_stream_bytes(size_t nbEle, int blockSize, int segments, int fastMode);

/* Device-pointer compressor.  d_data and d_out are device memory; stream is
 * a cudaStream_t (NULL: the legacy default stream).  segments <= 0
 * uses the default T.  Waits for the stream size, stores it in *outSize and
 * returns a status. */
int szp_gb300_compress_dev(int fastMode, const float *d_data, size_t nbEle, int errBoundMode, double absErrBound,
                           double relBoundRatio, int blockSize, int segments, unsigned char *d_out,
                           size_t out_capacity, size_t *outSize, void *stream);

/* As szp_gb300_compress_dev without waiting: the stream size is written to
 * d_outSize (device, 8 bytes) when the kernels finish.  Check errors with
 * szp_gb300_sync_status(). */
int szp_gb300_compress_dev_async(int fastMode, const float *d_data, size_t nbEle, int errBoundMode,
                                 double absErrBound, double relBoundRatio, int blockSize, int segments,
                                 unsigned char *d_out, size_t out_capacity, unsigned long long *d_outSize,
                                 void *stream);

/* float64 device-pointer compressor (waits for the size) and decompressor
 * (waits, returns the status); streams as szp_double_openmp_threadblock's. */
size_t szp_gb300_max_stream_bytes_f64(size_t nbEle, int blockSize, int segments, int fastMode);
int szp_gb300_compress_dev_f64(int fastMode, const double *d_data, size_t nbEle, int errBoundMode,
                               double absErrBound, double relBoundRatio, int blockSize, int segments,
                               unsigned char *d_out, size_t out_capacity, size_t *outSize, void *stream);
int szp_gb300_decompress_dev_f64(int fastMode, const unsigned char *d_bytes, size_t byteLength, size_t nbEle,
                                 int blockSize, int segments, double *d_out, void *stream);

/* Multidimensional Lorenzo variant (no reference entry point: the reference
 * predicts along the flattened array, SZp/example/test_multidim.cc).  A field
 * of nx*ny*nz floats, x fastest, in device memory, with an ABS or REL bound:
 * the stream is [nx][ny][nz] (u32 little-endian) followed by the fastmode1
 * stream (blockSize 32, `segments` segments of the flattened array) of the
 * codes q - q[j-1] - q[k-1] + q[j-1][k-1] (q: fastmode1's quantization codes,
 * neighbours outside the field 0), whose delta along x is the 3-D Lorenzo
 * residual.  Every value decompresses within eb, as fastmode1's do.  Waits;
 * the stream size goes to *outSize.  A 2-D field is nz = 1, a 1-D one
 * ny = nz = 1. */
size_t szp_gb300_lorenzo_max_stream_bytes(size_t nx, size_t ny, size_t nz, int segments);
int szp_gb300_lorenzo_compress_dev(const float *d_data, size_t nx, size_t ny, size_t nz, int errBoundMode,
                                   double absErrBound, double relBoundRatio, int segments, unsigned char *d_out,
                                   size_t out_capacity, size_t *outSize, void *stream);
/* Decompresses a Lorenzo stream of byteLength bytes into d_out; the dims and
 * segments must be those it was written with (other dims: SZP_GB300_EINVAL). */
int szp_gb300_lorenzo_decompress_dev(const unsigned char *d_bytes, size_t byteLength, size_t nx, size_t ny,
                                     size_t nz, int segments, float *d_out, void *stream);

/* Homomorphic sum of two device streams (the hZCCL use of fZ-light streams;
 * no reference entry point): both compressed from nbEle values with the same
 * error bound (identical eb header bytes), blockSize (8..256), segments and
 * fastMode, of dataType SZ_FLOAT or SZ_DOUBLE.  Writes to d_out the stream
 * whose quantization codes are the sums of a's and b's (wrapping int32; a
 * wrap is a notice, szp_gb300_last_notices), under the same header: it
 * decompresses to (q_a + q_b) * eb, within 2 * eb of the sum of the two
 * original fields.  Waits; stores the size in *outSize.  Streams with
 * different bounds give SZP_GB300_EINVAL. */
int szp_gb300_reduce_sum_dev(int fastMode, int dataType, const unsigned char *d_a, size_t lenA,
                             const unsigned char *d_b, size_t lenB, size_t nbEle, int blockSize, int segments,
                             unsigned char *d_out, size_t out_capacity, size_t *outSize, void *stream);

/* Device-pointer decompressor; asynchronous on stream.  d_bytes is a whole
 * stream of byteLength bytes in device memory. */
int szp_gb300_decompress_dev(int fastMode, const unsigned char *d_bytes, size_t byteLength, size_t nbEle,
                             int blockSize, int segments, float *d_out, void *stream);

/* As szp_gb300_decompress_dev, with the stream length read on the device
 * from d_byteLength (8 bytes, e.g. the size written by
 * szp_gb300_compress_dev_async); capacity bounds it.  Lets a compress ->
 * decompress pipeline run without a host round trip. */
int szp_gb300_decompress_dev_async(int fastMode, const unsigned char *d_bytes, size_t capacity,
                                   const unsigned long long *d_byteLength, size_t nbEle, int blockSize,
                                   int segments, float *d_out, void *stream);

/* Fastmode1 compressor that allocates nothing; no counterpart in the
 * reference.  For callers that cannot allocate device memory when they
 * compress (all GPU memory handed to their own pool, or a serving loop that
 * must not pay cudaMalloc's device-wide synchronisation): they pass device
 * buffers d_data and d_out, and the kernels' working memory is a static
 * device array of this library (about 136 KB per GPU that loads it, held until
 * the process exits).  At most 16384 tiles of 256 blocks (134,217,728 floats
 * at blockSize 32); larger inputs are rejected with SZP_GB300_EINVAL.  The
 * first call on a device looks up the array's device address (set-up).  All
 * calls share the array: calls that overlap on the GPU race.  Waits for the
 * result; *outSize gets the stream size (also when it exceeds out_capacity,
 * which returns SZP_GB300_ECAPACITY).  The stream equals szp_gb300_compress_dev's. */
int szp_gb300_compress_dev_noalloc(const float *d_data, size_t nbEle, int errBoundMode, double absErrBound,
                                   double relBoundRatio, int blockSize, int segments, unsigned char *d_out,
                                   size_t out_capacity, size_t *outSize, void *stream);

/* Waits for stream and returns the status of the device-side checks of the
 * calling thread's last calls (capacity, corrupt stream, timeouts). */
int szp_gb300_sync_status(void *stream);

/* Non-fatal notices of the last call: bit 0 set when some |x/eb| >= 2^31 or
 * x is NaN (undefined in the reference; quantized to INT32_MIN as its x86
 * build does). */
int szp_gb300_last_notices(void);

/* The 34-entry bit-count table, thr[k] = smallest m with
 * (int)log2f((float)m)+1 >= k, computed from this host's libm. */
void szp_gb300_bitcount_thresholds(uint32_t *thr34);

/* Runs the device bit-count rule on n device values (diagnostics). */
int szp_gb300_bitcount_probe(const uint32_t *d_max, uint8_t *d_bc, size_t n, void *stream);

/* Checks the device's bounded waits: one device thread waits on a barrier
 * that nothing completes, for at most limit_ns nanoseconds.  Returns
 * SZP_GB300_ETIMEOUT when the wait gave up as it must (the time waited in
 * *waited_ns); the device stays usable.  Every wait inside this library's
 * kernels gives up the same way, after about two seconds. */
int szp_gb300_wait_probe(unsigned long long limit_ns, unsigned long long *waited_ns);

/* Per-kernel timing with CUDA events on the launching stream.  When enabled,
 * szp_gb300_kernel_ms(slot) returns the duration of the last launch of:
 * 0 REL range, 1 compress, 2 decompress setup, 3 locate, 4 decode, 5 the
 * Lorenzo variant's codes pass, 6 its inverse sums (both of its passes). */
void szp_gb300_set_timing(int enable);
double szp_gb300_kernel_ms(int slot);

/* Sum of the durations (ms) of the launches of kernel `slot` timed since the
 * last call (up to 1024), and their number in *launches. */
double szp_gb300_kernel_time(int slot, int *launches);

/* Bytes a decompression CTA walks before its region to find the header
 * chain (-1: default).  Smaller values make the speculative walks fail more
 * often and exercise the repair paths; streams decode the same. */
void szp_gb300_set_locate_overlap(int bytes);

/* Nonzero: a single field's decode pipeline draws tile tickets instead of its
 * cooperative launch with a static tile order (the path it takes when a
 * cooperative launch is refused, e.g. on a partitioned GPU); streams decode
 * the same.  0 restores the default. */
void szp_gb300_set_decode_tickets(int on);

/* Chunks whose speculative header walk the last decompression of this
 * thread had to repair in order (statistics; -1 on error). */
int szp_gb300_last_repairs(void);

/* Number of kernels this library has launched in this process. */
unsigned long long szp_gb300_kernel_launches(void);

/* ---- batched fastmode1, blockSize 32 (no counterpart in the reference) ----
 * Many fields of uneven sizes and bounds go through one persistent launch per
 * stage (compress: range pass + tiles; decompress: header setup + locate +
 * decode), replayed as one CUDA graph.  Every field's stream is byte-identical
 * to szp_compress on that field alone with the same T.  All buffers are device
 * memory and must stay valid, and unchanged in size, for the batch's lifetime. */
typedef struct {
  const void *input;                       /* compress: float[nbEle]; decompress: the stream */
  size_t input_bytes;                      /* decompress: stream bytes readable at input */
  const unsigned long long *input_len_dev; /* decompress: optional device stream length
                                              (e.g. szp_gb300_batch_sizes_dev() + i), NULL = input_bytes */
  void *output;                            /* compress: stream buffer; decompress: float[nbEle] */
  size_t output_bytes;                     /* capacity of output in bytes */
  size_t nbEle;
  int errBoundMode;                        /* compress: ABS or REL */
  double absErrBound;
  double relBoundRatio;
} szp_gb300_field;

typedef struct szp_gb300_batch_s *szp_gb300_batch;

#define SZP_GB300_BATCH_COMPRESS 0
#define SZP_GB300_BATCH_DECOMPRESS 1
#define SZP_GB300_BATCH_AUTOTUNE 1 /* flags: time each tile size on the batch's inputs, keep the fastest */
#define SZP_GB300_BATCH_NO_GRAPH 2 /* flags: launch the stages directly instead of replaying a graph */
#define SZP_GB300_BATCH_ROUNDS(r) ((r) << 8) /* flags: fix the tile size (r = 1, 2 or 4) */

/* Builds the batch's tables on the device and captures its graph; T as for
 * szp_compress (segments <= 0: OpenMP's thread count). */
int szp_gb300_batch_create(szp_gb300_batch *out, int direction, const szp_gb300_field *fields, int nfields,
                           int blockSize, int segments, int flags);
/* Queues one run on a stream (NULL = legacy default stream). */
int szp_gb300_batch_run(szp_gb300_batch b, void *stream);
/* Waits for the last run; per-field stream sizes (compress) and statuses
 * (SZP_GB300_*), either pointer may be NULL.  Returns the first failure. */
int szp_gb300_batch_sync(szp_gb300_batch b, unsigned long long *sizes, int *status);
/* Device array of the per-field stream sizes written by a compress run. */
const unsigned long long *szp_gb300_batch_sizes_dev(szp_gb300_batch b);
/* Tile size in use: tiles of 64 * rounds blocks (1, 2 or 4). */
int szp_gb300_batch_tile_rounds(szp_gb300_batch b);
void szp_gb300_batch_destroy(szp_gb300_batch b);

/* ---- request server: continuous batching on device-resident data (no
 * counterpart in the reference) ----
 * Requests are admitted in arrival order while their results fit the HBM
 * budget, launched in groups (one compress batch + one decompress batch per
 * group) on up to `lanes` streams at once, and keep their results on the
 * device until released.  Every result is byte-identical to the single-field
 * calls on the same input.  blockSize is 32. */
typedef struct {
  int op;                 /* SZP_GB300_BATCH_COMPRESS or SZP_GB300_BATCH_DECOMPRESS */
  const void *input;      /* device: float[nbEle] (compress) or a stream (decompress) */
  size_t input_bytes;     /* decompress: stream bytes */
  size_t nbEle;
  int errBoundMode;       /* compress: ABS or REL */
  double absErrBound;
  double relBoundRatio;
  double arrival;         /* server-clock seconds; < 0: the submission time */
} szp_gb300_request;

typedef struct {
  unsigned long long id;
  int status;             /* SZP_GB300_* */
  void *output;           /* device: the stream or float[nbEle], valid until released */
  size_t output_bytes;    /* stream bytes, or 4 * nbEle */
  double arrival, admitted, done; /* server-clock seconds */
} szp_gb300_result;

typedef struct {
  size_t hbm_budget;      /* device bytes for results (one arena) */
  int max_batch;          /* requests per group at most */
  int lanes;              /* groups in flight at once, 1..16 */
  int segments;           /* T of every stream; <= 0: OpenMP's thread count */
  int tile_rounds;        /* 1, 2 or 4; 0: chosen per group from the request sizes */
} szp_gb300_server_config;

typedef struct {
  unsigned long long requests, bytes, queued, in_flight, memory_used, memory_peak;
} szp_gb300_server_stats;

typedef struct szp_gb300_server_s *szp_gb300_server;

int szp_gb300_server_create(szp_gb300_server *out, const szp_gb300_server_config *cfg);
/* Queues n requests; ids[i] receives each one's id (ids may be NULL). */
int szp_gb300_server_submit(szp_gb300_server s, const szp_gb300_request *reqs, int n, unsigned long long *ids);
/* Results finished since the last call, at most max; returns how many. */
int szp_gb300_server_completed(szp_gb300_server s, szp_gb300_result *res, int max);
/* Blocks until request id has finished; returns its status. */
int szp_gb300_server_wait(szp_gb300_server s, unsigned long long id, szp_gb300_result *res);
/* Frees a finished request's result. */
int szp_gb300_server_release(szp_gb300_server s, unsigned long long id);
/* Blocks until nothing is queued or running. */
int szp_gb300_server_drain(szp_gb300_server s);
int szp_gb300_server_get_stats(szp_gb300_server s, szp_gb300_server_stats *st);
double szp_gb300_server_clock(szp_gb300_server s);
void szp_gb300_server_destroy(szp_gb300_server s);

#ifdef __cplusplus
}
#endif

#endif /* SZP_GB300_H */
