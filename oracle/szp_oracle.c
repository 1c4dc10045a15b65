/*
 * szp_oracle.c -- CPU restatement of SZp's fastmode1 (SZP_NONRANDOMACCESS) and
 * fastmode2 (SZP_RANDOMACCESS) float32 codec.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA library is
 * checked against; it is also the "port" CPU baseline timed by bench.py.  The
 * product library (szp_gb300/) never links, loads or calls it.
 *
 * Parity is pinned: tests/test_oracle_golden.py checks every function here
 * byte-for-byte against fixtures written by the reference library itself
 * (tests/golden/make_golden.py builds and runs it), and, when the reference
 * sources are present, against the freshly built reference on random inputs.
 *
 * Stream layout restated (fastmode1, SZp/src/szp_float.cc:148-309):
 *   [eb : float32, big-endian]                       szp_float.cc:164, szp_CompressionToolkit.h:520-527
 *   [off: size_t x T, native little-endian]          szp_float.cc:280-289
 *   [segment 0] ... [segment T-1]                    szp_float.cc:291
 * segment t covers elements [t*floor(n/T), (t+1)*floor(n/T)), the last one
 * takes the remainder (szp_float.cc:186,194-199).  A non-empty segment is
 *   [seed: int32 LE = q(x[lo])] {block}*            szp_float.cc:208-213
 * and its blocks start at lo+1, lo+1+L, ... (last one may be shorter).
 * block = [bc: u8]                                   szp_float.cc:253-262
 *         if bc > 0: [sign bits MSB-first, ceil(m/8) bytes]  szp_TypeManager.cc:820-844
 *                    [payload]                        szp_TypeManager.cc:13-94
 * payload = m x (bc/8) bytes holding (v >> bc%8) little-endian, then the low
 * bc%8 bits of every v as one MSB-first bit string (ceil(m*(bc%8)/8) bytes).
 *
 * fastmode2 (szp_float.cc:752-1076): segments as above, but every block starts
 * at lo + k*L and carries its own int32 seed; the diffs cover the m-1 elements
 * after the seed.
 *
 * float64 (SZp/src/szp_double.cc, szpd_double.cc): the same segments and
 * blocks; eb is a big-endian double (8 bytes, szp_double.cc:164 and
 * szp_CompressionToolkit.h:530-546), so the offsets start at byte 8;
 * q = (int)(x * (1/eb)) with a double product (szp_double.cc:180,209,228)
 * and x' = (double)q * eb (szpd_double.cc:67,86,112).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define SZO_OK 0
#define SZO_ERR_ARG -1
#define SZO_ERR_CAP -2
#define SZO_ERR_STREAM -3
#define SZO_ERR_NOMEM -4

/* (int)log2f((float)max) + 1 for max > 0, else 0 -- szp_float.cc:253-262.
 * The float conversion rounds to nearest and libm's log2f rounds its result,
 * which makes the value one larger than the true bit width just below 2^k
 * for k >= 21 (up to 33). */
int szo_bitcount(uint32_t max)
{
    if (max == 0) return 0;
    return (int)(log2f((float)max)) + 1;
}

/* q = (int)((double)x * (double)(1.0f/eb)) -- szp_float.cc:185,209,228.
 * The product of two floats is exact in double, the cast truncates toward
 * zero.  Out of range and NaN are undefined in C; x86-64 (cvttsd2si) returns
 * INT32_MIN, which is what this restatement pins so that it gives the same
 * answer on every host. */
static inline int32_t quantize(float x, double inv)
{
    double p = (double)x * inv;
    if (p > -2147483649.0 && p < 2147483648.0) return (int32_t)p;
    return INT32_MIN;
}

/* q = (int)(x * inv) for double x, szp_double.cc:209,228: the double product
 * rounds to nearest; out of range and NaN give INT32_MIN as above. */
static inline int32_t quantize_d(double x, double inv)
{
    double p = x * inv;
    if (p > -2147483649.0 && p < 2147483648.0) return (int32_t)p;
    return INT32_MIN;
}

/* Float results that are NaN follow x86 SSE, the platform the reference's
 * fixtures were made on: a NaN operand propagates (quieted); an invalid
 * operation (0*inf, inf-inf) gives the default NaN 0xFFC00000.  aarch64 would
 * give +0x7FC00000 there, so the restatement states the rule instead of
 * inheriting the host's. */
static inline float x86_nan_fix(float r, float a, float b)
{
    if (r == r) return r;
    uint32_t u;
    if (a != a) memcpy(&u, &a, 4);
    else if (b != b) memcpy(&u, &b, 4);
    else u = 0xFFC00000u;
    u |= 0x00400000u;
    memcpy(&r, &u, 4);
    return r;
}

/* (float)q * eb, szpd_float.cc:67,86,112 */
static inline float dequant(int32_t q, float eb)
{
    float f = (float)q;
    return x86_nan_fix(f * eb, f, eb);
}

/* x86 SSE NaN rule for double results: a NaN operand propagates quieted, an
 * invalid operation gives the default NaN 0xFFF8000000000000. */
static inline double x86_nan_fix_d(double r, double a, double b)
{
    if (r == r) return r;
    uint64_t u;
    if (a != a) memcpy(&u, &a, 8);
    else if (b != b) memcpy(&u, &b, 8);
    else u = 0xFFF8000000000000ull;
    u |= 0x0008000000000000ull;
    memcpy(&r, &u, 8);
    return r;
}

/* (double)q * eb, szpd_double.cc:67,86,112 */
static inline double dequant_d(int32_t q, double eb)
{
    double f = (double)q;
    return x86_nan_fix_d(f * eb, f, eb);
}

/* Array kinds of the codec bodies: float data, double data, or the int32
 * quantization codes themselves (the reduction below) under a float or a
 * double stream header. */
enum { KIND_FLOAT = 0, KIND_DOUBLE = 1, KIND_Q_F = 2, KIND_Q_D = 3 };
static inline size_t kind_hb(int kind) { return (kind == KIND_DOUBLE || kind == KIND_Q_D) ? 8 : 4; }

/* Element i of the input, quantized (codes are taken as they are). */
static inline int32_t q_at(const void *x, int kind, size_t i, double inv)
{
    if (kind == KIND_DOUBLE) return quantize_d(((const double *)x)[i], inv);
    if (kind == KIND_FLOAT) return quantize(((const float *)x)[i], inv);
    return ((const int32_t *)x)[i];
}

/* y[i] = dequantized q (or q itself for a code array). */
static inline void put_y(void *y, int kind, size_t i, int32_t q, double eb)
{
    if (kind == KIND_DOUBLE) ((double *)y)[i] = dequant_d(q, eb);
    else if (kind == KIND_FLOAT) ((float *)y)[i] = dequant(q, (float)eb);
    else ((int32_t *)y)[i] = q;
}

static inline void put_u32le(unsigned char *p, uint32_t v)
{
    p[0] = (unsigned char)v; p[1] = (unsigned char)(v >> 8);
    p[2] = (unsigned char)(v >> 16); p[3] = (unsigned char)(v >> 24);
}
static inline uint32_t get_u32le(const unsigned char *p)
{
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
static inline void put_u64le(unsigned char *p, uint64_t v)
{
    for (int i = 0; i < 8; i++) p[i] = (unsigned char)(v >> (8 * i));
}
static inline uint64_t get_u64le(const unsigned char *p)
{
    uint64_t v = 0;
    for (int i = 0; i < 8; i++) v |= (uint64_t)p[i] << (8 * i);
    return v;
}

/* Bytes of one encoded block of m elements with bit count bc. */
static inline size_t block_bytes(size_t m, int bc)
{
    if (bc == 0) return 1;
    size_t B = (size_t)(bc / 8), r = (size_t)(bc % 8);
    return 1 + (m + 7) / 8 + B * m + (r * m + 7) / 8;
}

/* Write one block (header, sign bits, byte planes, remainder bit string) for
 * m magnitudes v[] and sign flags s[]; returns bytes written.  Follows
 * szp_float.cc:253-274 with szp_TypeManager.cc:13-94,122-434,820-844. */
static size_t put_block(unsigned char *o, const uint32_t *v, const unsigned char *s, size_t m, uint32_t max)
{
    int bc = szo_bitcount(max);
    o[0] = (unsigned char)bc;
    if (bc == 0) return 1;
    unsigned char *p = o + 1;
    size_t nsign = (m + 7) / 8;
    memset(p, 0, nsign);
    for (size_t j = 0; j < m; j++)
        if (s[j]) p[j >> 3] |= (unsigned char)(0x80u >> (j & 7));
    p += nsign;
    int B = bc / 8, r = bc % 8;
    for (size_t j = 0; j < m; j++) {
        uint32_t hi = v[j] >> r;
        for (int b = 0; b < B; b++) p[j * B + b] = (unsigned char)(hi >> (8 * b));
    }
    p += (size_t)B * m;
    if (r) {
        size_t nrem = (r * m + 7) / 8;
        memset(p, 0, nrem);
        uint32_t mask = (1u << r) - 1u;
        for (size_t j = 0; j < m; j++) {
            uint32_t lo = v[j] & mask;
            for (int b = 0; b < r; b++) {
                size_t bit = j * (size_t)r + (size_t)b; /* MSB of the r bits first */
                if ((lo >> (r - 1 - b)) & 1u) p[bit >> 3] |= (unsigned char)(0x80u >> (bit & 7));
            }
        }
    }
    return block_bytes(m, bc);
}

/* Read one block of m elements at i; fills v[] and s[]; returns bytes
 * consumed or 0 on a bad header.  Mirrors szpd_float.cc:79-117 with
 * szp_TypeManager.cc:436-517,902-944. */
static size_t get_block(const unsigned char *i, const unsigned char *end, uint32_t *v, unsigned char *s, size_t m)
{
    if (i >= end) return 0;
    int bc = i[0];
    if (bc > 33) return 0;
    size_t nb = block_bytes(m, bc);
    if ((size_t)(end - i) < nb) return 0;
    if (bc == 0) {
        for (size_t j = 0; j < m; j++) { v[j] = 0; s[j] = 0; }
        return 1;
    }
    const unsigned char *p = i + 1;
    for (size_t j = 0; j < m; j++) s[j] = (p[j >> 3] >> (7 - (j & 7))) & 1u;
    p += (m + 7) / 8;
    int B = bc / 8, r = bc % 8;
    for (size_t j = 0; j < m; j++) {
        uint32_t hi = 0;
        for (int b = 0; b < B; b++) hi |= (uint32_t)p[j * B + b] << (8 * b);
        v[j] = B ? (hi << r) : 0;
    }
    p += (size_t)B * m;
    for (size_t j = 0; j < m && r; j++) {
        uint32_t lo = 0;
        for (int b = 0; b < r; b++) {
            size_t bit = j * (size_t)r + (size_t)b;
            lo = (lo << 1) | ((p[bit >> 3] >> (7 - (bit & 7))) & 1u);
        }
        v[j] |= lo;
    }
    return nb;
}

/* Segment bounds, szp_float.cc:186,194-199 and szpd_float.cc:40-47. */
static inline void seg_bounds(size_t n, int T, int t, size_t *lo, size_t *hi)
{
    size_t tsz = n / (size_t)T;
    *lo = (size_t)t * tsz;
    *hi = (t == T - 1) ? n : (size_t)(t + 1) * tsz;
}

/* Upper bound of the stream size for (n, L, T) in either mode (float). */
size_t szo_max_stream_bytes(size_t n, int L, int T, int mode)
{
    if (L <= 0 || T <= 0) return 0;
    size_t full = block_bytes((size_t)L, 33);
    size_t nblk = n / (size_t)L + (size_t)T + 1;
    size_t per = (mode == 2) ? 4 : 0;
    return 4 + 8 * (size_t)T + 4 * (size_t)T + nblk * (full + per);
}

/* The same for double data (8-byte eb). */
size_t szo_max_stream_bytes_d(size_t n, int L, int T, int mode)
{
    size_t b = szo_max_stream_bytes(n, L, T, mode);
    return b ? b + 4 : 0;
}

/* Encode segment [lo,hi) into o; returns bytes.  Fastmode1 loop,
 * szp_float.cc:206-275. */
static size_t encode_segment_fm1(const void *x, int dbl, size_t lo, size_t hi, double inv, size_t L,
                                 unsigned char *o, uint32_t *v, unsigned char *s)
{
    if (lo >= hi) return 0;
    size_t w = 0;
    int32_t prior = q_at(x, dbl, lo, inv);
    put_u32le(o, (uint32_t)prior);
    w += 4;
    for (size_t i = lo + 1; i < hi; i += L) {
        size_t m = (i + L > hi) ? hi - i : L;
        uint32_t max = 0;
        for (size_t j = 0; j < m; j++) {
            int32_t cur = q_at(x, dbl, i + j, inv);
            uint32_t d = (uint32_t)cur - (uint32_t)prior; /* wrapping, as compiled x86 code does */
            prior = cur;
            s[j] = (int32_t)d < 0;
            v[j] = s[j] ? 0u - d : d;
            if (v[j] > max) max = v[j];
        }
        w += put_block(o + w, v, s, m, max);
    }
    return w;
}

/* Fastmode2 segment: every block restarts from its own seed,
 * szp_float.cc:812-864. */
static size_t encode_segment_fm2(const void *x, int dbl, size_t lo, size_t hi, double inv, size_t L,
                                 unsigned char *o, uint32_t *v, unsigned char *s)
{
    size_t w = 0;
    for (size_t i = lo; i < hi; i += L) {
        size_t m = (i + L > hi) ? hi - i : L;
        int32_t prior = q_at(x, dbl, i, inv);
        put_u32le(o + w, (uint32_t)prior);
        w += 4;
        uint32_t max = 0;
        for (size_t j = 0; j + 1 < m; j++) {
            int32_t cur = q_at(x, dbl, i + j + 1, inv);
            uint32_t d = (uint32_t)cur - (uint32_t)prior;
            prior = cur;
            s[j] = (int32_t)d < 0;
            v[j] = s[j] ? 0u - d : d;
            if (v[j] > max) max = v[j];
        }
        w += put_block(o + w, v, s, m - 1, max);
    }
    return w;
}

/* Compressor body for an array of the given kind (float data: eb header 4
 * bytes; double data: 8); inv and the header bytes come from the caller. */
static int compress_any(const void *x, int dbl, size_t n, double inv, const unsigned char *ebb, int L, int T,
                        int mode, unsigned char *out, size_t cap, size_t *out_size)
{
    if (L <= 0 || T <= 0 || (mode != 1 && mode != 2) || !out || !out_size) return SZO_ERR_ARG;
    const size_t hb = kind_hb(dbl);
    size_t head = hb + 8 * (size_t)T;
    if (cap < head) return SZO_ERR_CAP;
    memcpy(out, ebb, hb);

    size_t *sz = (size_t *)calloc((size_t)T, sizeof(size_t));
    unsigned char **buf = (unsigned char **)calloc((size_t)T, sizeof(unsigned char *));
    if (!sz || !buf) { free(sz); free(buf); return SZO_ERR_NOMEM; }
    int fail = 0;
#pragma omp parallel for schedule(static, 1) num_threads(T)
    for (int t = 0; t < T; t++) {
        size_t lo, hi;
        seg_bounds(n, T, t, &lo, &hi);
        size_t len = hi > lo ? hi - lo : 0;
        size_t nblk = len / (size_t)L + 2;
        size_t bound = 4 + nblk * (block_bytes((size_t)L, 33) + 4);
        buf[t] = (unsigned char *)malloc(bound);
        uint32_t *v = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)L);
        unsigned char *s = (unsigned char *)malloc((size_t)L);
        if (!buf[t] || !v || !s) {
#pragma omp atomic write
            fail = 1;
        } else if (mode == 1) {
            sz[t] = encode_segment_fm1(x, dbl, lo, hi, inv, (size_t)L, buf[t], v, s);
        } else {
            sz[t] = encode_segment_fm2(x, dbl, lo, hi, inv, (size_t)L, buf[t], v, s);
        }
        free(v);
        free(s);
    }
    int rc = SZO_OK;
    if (fail) rc = SZO_ERR_NOMEM;
    size_t total = head;
    if (rc == SZO_OK) {
        size_t off = 0;
        for (int t = 0; t < T; t++) { put_u64le(out + hb + 8 * (size_t)t, off); off += sz[t]; }
        total = head + off;
        if (total > cap) rc = SZO_ERR_CAP;
    }
    if (rc == SZO_OK) {
        size_t off = head;
        for (int t = 0; t < T; t++) { memcpy(out + off, buf[t], sz[t]); off += sz[t]; }
        *out_size = total;
    }
    for (int t = 0; t < T; t++) free(buf[t]);
    free(buf);
    free(sz);
    return rc;
}

/* Full compressor with explicit segment count T (the reference's OpenMP
 * thread count).  mode 1 = fastmode1, 2 = fastmode2.  Writes into out
 * (capacity cap) and returns SZO_OK or an error. */
int szo_compress(const float *x, size_t n, float eb, int L, int T, int mode,
                 unsigned char *out, size_t cap, size_t *out_size)
{
    /* float division stored in a double, szp_float.cc:185 */
    double inv = (double)(1.0f / eb);
    unsigned char ebb[4], be[4];
    memcpy(ebb, &eb, 4);
    be[0] = ebb[3]; be[1] = ebb[2]; be[2] = ebb[1]; be[3] = ebb[0];
    return compress_any(x, 0, n, inv, be, L, T, mode, out, cap, out_size);
}

/* Double compressor, szp_double.cc:149-309 (fastmode1), :759-920 (fastmode2):
 * inv = 1/eb in double (szp_double.cc:180). */
int szo_compress_d(const double *x, size_t n, double eb, int L, int T, int mode,
                   unsigned char *out, size_t cap, size_t *out_size)
{
    double inv = 1.0 / eb;
    unsigned char ebb[8], be[8];
    memcpy(ebb, &eb, 8);
    for (int i = 0; i < 8; i++) be[i] = ebb[7 - i];
    return compress_any(x, 1, n, inv, be, L, T, mode, out, cap, out_size);
}

/* Decoder for one fastmode1 segment, szpd_float.cc:59-118. */
static int decode_segment_fm1(const unsigned char *p, const unsigned char *end, size_t lo, size_t hi,
                              double eb, size_t L, void *y, int dbl, uint32_t *v, unsigned char *s)
{
    if (lo >= hi) return SZO_OK;
    if (end - p < 4) return SZO_ERR_STREAM;
    int32_t prior = (int32_t)get_u32le(p);
    p += 4;
    put_y(y, dbl, lo, prior, eb);
    for (size_t i = lo + 1; i < hi; i += L) {
        size_t m = (i + L > hi) ? hi - i : L;
        size_t nb = get_block(p, end, v, s, m);
        if (!nb) return SZO_ERR_STREAM;
        p += nb;
        for (size_t j = 0; j < m; j++) {
            uint32_t d = s[j] ? 0u - v[j] : v[j];
            prior = (int32_t)((uint32_t)prior + d);
            put_y(y, dbl, i + j, prior, eb);
        }
    }
    return SZO_OK;
}

/* Decoder for one fastmode2 segment, szpd_float.cc:425-637. */
static int decode_segment_fm2(const unsigned char *p, const unsigned char *end, size_t lo, size_t hi,
                              double eb, size_t L, void *y, int dbl, uint32_t *v, unsigned char *s)
{
    for (size_t i = lo; i < hi; i += L) {
        size_t m = (i + L > hi) ? hi - i : L;
        if (end - p < 4) return SZO_ERR_STREAM;
        int32_t prior = (int32_t)get_u32le(p);
        p += 4;
        put_y(y, dbl, i, prior, eb);
        /* a one-element block has no header byte on the decode side, although
         * the encoder wrote a 0 for it (szpd_float.cc:483 vs szp_float.cc:848).
         * With blockSize > 1 that is only a segment's last block, so nothing
         * shifts; with blockSize 1 every block is one, and the reads fall one
         * byte further behind per block, as in the reference. */
        if (m == 1) continue;
        size_t nb = get_block(p, end, v, s, m - 1);
        if (!nb) return SZO_ERR_STREAM;
        p += nb;
        for (size_t j = 0; j + 1 < m; j++) {
            uint32_t d = s[j] ? 0u - v[j] : v[j];
            prior = (int32_t)((uint32_t)prior + d);
            put_y(y, dbl, i + j + 1, prior, eb);
        }
    }
    return SZO_OK;
}

/* Decompressor body: stream (len bytes, including the eb header of the
 * kind's width), explicit T.  Validates offsets against len. */
static int decompress_any(const unsigned char *stream, size_t len, size_t n, int L, int T, int mode, double eb,
                          int dbl, void *y)
{
    const size_t hb = kind_hb(dbl);
    size_t head = hb + 8 * (size_t)T;
    if (len < head) return SZO_ERR_STREAM;
    const unsigned char *data = stream + head;
    const unsigned char *end = stream + len;
    int rc = SZO_OK;
#pragma omp parallel for schedule(static, 1) num_threads(T)
    for (int t = 0; t < T; t++) {
        size_t lo, hi;
        seg_bounds(n, T, t, &lo, &hi);
        uint64_t off = get_u64le(stream + hb + 8 * (size_t)t);
        int r = SZO_OK;
        if (lo < hi && off > (uint64_t)(end - data)) r = SZO_ERR_STREAM;
        uint32_t *v = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)L);
        unsigned char *s = (unsigned char *)malloc((size_t)L);
        if (!v || !s) r = SZO_ERR_NOMEM;
        if (r == SZO_OK) {
            if (mode == 1) r = decode_segment_fm1(data + off, end, lo, hi, eb, (size_t)L, y, dbl, v, s);
            else r = decode_segment_fm2(data + off, end, lo, hi, eb, (size_t)L, y, dbl, v, s);
        }
        free(v);
        free(s);
        if (r != SZO_OK) {
#pragma omp critical
            rc = r;
        }
    }
    return rc;
}

/* Full decompressor: stream (len bytes, including the 4-byte eb header),
 * explicit T.  Validates offsets against len. */
int szo_decompress(const unsigned char *stream, size_t len, size_t n, int L, int T, int mode, float *y)
{
    if (L <= 0 || T <= 0 || (mode != 1 && mode != 2) || !stream || (!y && n)) return SZO_ERR_ARG;
    if (len < 4) return SZO_ERR_STREAM;
    unsigned char ebb[4] = {stream[3], stream[2], stream[1], stream[0]};
    float eb;
    memcpy(&eb, ebb, 4);
    return decompress_any(stream, len, n, L, T, mode, (double)eb, 0, y);
}

/* Double decompressor, szpd_double.cc:23-128 (fastmode1), :431-535 (fastmode2). */
int szo_decompress_d(const unsigned char *stream, size_t len, size_t n, int L, int T, int mode, double *y)
{
    if (L <= 0 || T <= 0 || (mode != 1 && mode != 2) || !stream || (!y && n)) return SZO_ERR_ARG;
    if (len < 8) return SZO_ERR_STREAM;
    unsigned char ebb[8];
    for (int i = 0; i < 8; i++) ebb[i] = stream[7 - i];
    double eb;
    memcpy(&eb, ebb, 8);
    return decompress_any(stream, len, n, L, T, mode, eb, 1, y);
}

/* Homomorphic sum of two streams of the same eb, blockSize, T and mode
 * (not a reference function: the hZCCL use of fZ-light streams).  The result
 * is the stream whose quantization codes are qa[i] + qb[i] (wrapping int32
 * arithmetic, as the codecs' deltas wrap), under a's eb header: it
 * decompresses to (qa[i] + qb[i]) * eb.  hb = 4 for float streams, 8 for
 * double streams.  Headers that differ are an argument error. */
int szo_reduce_sum(const unsigned char *a, size_t alen, const unsigned char *b, size_t blen, size_t n, int L, int T,
                   int mode, int hb, unsigned char *out, size_t cap, size_t *out_size)
{
    if (L <= 0 || T <= 0 || (mode != 1 && mode != 2) || (hb != 4 && hb != 8) || !a || !b || !out || !out_size)
        return SZO_ERR_ARG;
    if (alen < (size_t)hb || blen < (size_t)hb) return SZO_ERR_STREAM;
    if (memcmp(a, b, (size_t)hb) != 0) return SZO_ERR_ARG;
    const int kind = hb == 8 ? KIND_Q_D : KIND_Q_F;
    int32_t *qa = (int32_t *)malloc(sizeof(int32_t) * (n ? n : 1));
    int32_t *qb = (int32_t *)malloc(sizeof(int32_t) * (n ? n : 1));
    int rc = (qa && qb) ? SZO_OK : SZO_ERR_NOMEM;
    if (rc == SZO_OK) rc = decompress_any(a, alen, n, L, T, mode, 0.0, kind, qa);
    if (rc == SZO_OK) rc = decompress_any(b, blen, n, L, T, mode, 0.0, kind, qb);
    if (rc == SZO_OK) {
        for (size_t i = 0; i < n; i++) qa[i] = (int32_t)((uint32_t)qa[i] + (uint32_t)qb[i]);
        rc = compress_any(qa, kind, n, 0.0, a, L, T, mode, out, cap, out_size);
    }
    free(qa);
    free(qb);
    return rc;
}

/* REL bound: serial min/max and (max-min)*(float)rel in float,
 * SZp/src/szp.cc:33-48. */
float szo_rel_bound(const float *x, size_t n, double rel)
{
    if (n == 0) return 0.0f;
    float mn = x[0], mx = x[0];
    for (size_t i = 0; i < n; i++) {
        float v = x[i];
        if (mn > v) mn = v;
        else if (mx < v) mx = v;
    }
    float range = x86_nan_fix(mx - mn, mx, mn);
    float r = (float)rel;
    return x86_nan_fix(range * r, range, r);
}

/* REL bound for double data: serial min/max and (max-min)*rel in double,
 * SZp/src/szp.cc:77-89. */
double szo_rel_bound_d(const double *x, size_t n, double rel)
{
    if (n == 0) return 0.0;
    double mn = x[0], mx = x[0];
    for (size_t i = 0; i < n; i++) {
        double v = x[i];
        if (mn > v) mn = v;
        else if (mx < v) mx = v;
    }
    double range = x86_nan_fix_d(mx - mn, mx, mn);
    return x86_nan_fix_d(range * rel, range, rel);
}

/* The 34 bit-count thresholds: thr[k] = smallest m >= 1 with
 * szo_bitcount(m) >= k, k = 1..33 (thr[0] = 0).  Found by bisection, which
 * is valid because bitcount is non-decreasing (checked exhaustively by the
 * test suite). */
void szo_bitcount_thresholds(uint32_t *thr)
{
    thr[0] = 0;
    for (int k = 1; k <= 33; k++) {
        uint64_t a = 1, b = 0xFFFFFFFFull; /* find smallest m in [a,b] with bc(m) >= k */
        if (szo_bitcount((uint32_t)b) < k) { thr[k] = 0xFFFFFFFFu; continue; }
        while (a < b) {
            uint64_t mid = (a + b) / 2;
            if (szo_bitcount((uint32_t)mid) >= k) b = mid; else a = mid + 1;
        }
        thr[k] = (uint32_t)a;
    }
}

/* Exhaustive check that bitcount is non-decreasing over [1, 2^32) and agrees
 * with the thresholds; returns the number of disagreements.  Used by tests. */
uint64_t szo_bitcount_verify(const uint32_t *thr)
{
    uint64_t bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(static)
    for (int64_t hiw = 0; hiw < 65536; hiw++) {
        for (uint32_t low = 0; low < 65536; low++) {
            uint32_t m = ((uint32_t)hiw << 16) | low;
            if (m == 0) continue;
            int bc = szo_bitcount(m);
            int k = 32 - __builtin_clz(m);
            int want = k + (k < 33 && m >= thr[k + 1] ? 1 : 0);
            if (bc != want) bad++;
        }
    }
    return bad;
}

int szo_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* The `total_memaccess` tallies returned by the reference's single-thread
 * _record entry points, restated step by step over a T = 1 fastmode1 stream
 * (the stream the matching single-thread compressor writes).  The counts are
 * the reference's own bookkeeping of the bytes each statement touches, not a
 * measurement.  q = 4 for float data, 8 for double data.
 *
 * Compressor, szp_float.cc:607-750 (szp_double.cc:613-756 for double data):
 *   8 for *outSize (:622); for n > 0 the seed: q read + 2*4 (:651,653);
 *   per element q read + 1 + 4 for the temp arrays (:672,695); per block
 *   1 for the bit count (:700,708), and for a non-zero block the m sign
 *   reads, the sign bytes, the 4m magnitude reads and the payload bytes
 *   (:713-722); at the end 8 + 8 + 3*8 + 2*8 + 2 * segment bytes (:728-739).
 * Decompressor, szpd_float.cc:216-318 (szpd_double.cc:219-321):
 *   8 for the offset (:239); for n > 0 2*4 for the seed + 2q for x'[0]
 *   (:246,251); per block 1 for the bit count (:266); a zero block 2q per
 *   element (:275); a non-zero block its sign bytes + m, its payload bytes +
 *   4m, and 1 + 4 + 2q per element (:283-309).
 * Returns 0 for a stream that does not parse. */
uint64_t szo_record_compress(const unsigned char *stream, size_t len, size_t n, int L, int dbl)
{
    if (L <= 0) return 0;
    const uint64_t q = dbl ? 8 : 4;
    const size_t hb = dbl ? 8 : 4;
    uint64_t acc = 8;
    if (len < hb + 8) return 0;
    const unsigned char *p = stream + hb + 8, *end = stream + len;
    uint64_t seg = 0;
    if (n > 0) {
        acc += q + 8;
        p += 4;
        seg += 4;
    }
    for (size_t i = 1; i < n; i += (size_t)L) {
        size_t m = (i + (size_t)L > n) ? n - i : (size_t)L;
        if (p >= end || p[0] > 33) return 0;
        int bc = p[0];
        size_t nb = block_bytes(m, bc);
        acc += (q + 5) * m;               /* each element: x read, temp sign, temp magnitude */
        acc += 1;                         /* the bit-count byte */
        if (bc) {
            size_t nsign = (m + 7) / 8;
            acc += m + nsign;             /* temp signs read, sign bytes written */
            acc += 4 * m + (nb - 1 - nsign); /* magnitudes read, payload written */
        }
        p += nb;
        seg += nb;
    }
    if (p > end) return 0;
    acc += 8 + 8 + 3 * 8 + 2 * 8;
    acc += 2 * seg;
    return acc;
}

uint64_t szo_record_decompress(const unsigned char *stream, size_t len, size_t n, int L, int dbl)
{
    if (L <= 0) return 0;
    const uint64_t q = dbl ? 8 : 4;
    const size_t hb = dbl ? 8 : 4;
    uint64_t acc = 8;
    if (len < hb + 8) return 0;
    const unsigned char *p = stream + hb + 8, *end = stream + len;
    if (n > 0) {
        acc += 2 * 4 + 2 * q;
        p += 4;
    }
    for (size_t i = 1; i < n; i += (size_t)L) {
        size_t m = (i + (size_t)L > n) ? n - i : (size_t)L;
        if (p >= end || p[0] > 33) return 0;
        int bc = p[0];
        size_t nb = block_bytes(m, bc);
        acc += 1;
        if (bc == 0) {
            acc += 2 * q * m;
        } else {
            size_t nsign = (m + 7) / 8;
            acc += nsign + m;                   /* sign bytes read, temp signs written */
            acc += (nb - 1 - nsign) + 4 * m;    /* payload read, temp magnitudes written */
            acc += (1 + 4 + 2 * q) * m;         /* per element: temps read, x' stored */
        }
        p += nb;
    }
    if (p > end) return 0;
    return acc;
}

/* --------------------------------------------------------------------------
 * Multidimensional Lorenzo variant.  Not a reference function: the reference
 * predicts along the flattened array only (its example/test_multidim.cc
 * flattens the dimensions), so this defines its own stream, and its parity is
 * pinned by its round trips and by the CUDA library agreeing with this
 * restatement byte for byte.
 *
 * For a field of nx*ny*nz floats (x fastest) with fastmode1's codes q
 * (szp_float.cc:185,209,228), the stream packs the codes
 *     r = q - q[j-1] - q[k-1] + q[j-1][k-1]      (neighbours outside are 0)
 * with fastmode1 (blockSize 32, T segments of the flattened array); the 1-D
 * delta fastmode1 takes along x turns r into the 3-D Lorenzo residual
 * q - (q[i-1] + q[j-1] + q[k-1] - q[i-1][j-1] - q[i-1][k-1] - q[j-1][k-1]
 * + q[i-1][j-1][k-1]) inside the field.  Codes wrap as int32.
 * Stream: [nx][ny][nz] as u32 little-endian, then the fastmode1 stream of r
 * (float eb header).  Decompression decodes r, sums it along y and along z,
 * and dequantizes like fastmode1.
 * -------------------------------------------------------------------------- */
#define SZO_LORENZO_HEAD 12

size_t szo_lorenzo_max_stream_bytes(size_t nx, size_t ny, size_t nz, int T)
{
    return SZO_LORENZO_HEAD + szo_max_stream_bytes(nx * ny * nz, 32, T, 1);
}

int szo_lorenzo_compress(const float *x, size_t nx, size_t ny, size_t nz, float eb, int T, unsigned char *out,
                         size_t cap, size_t *out_size)
{
    if (!out || !out_size || T <= 0 || nx > UINT32_MAX || ny > UINT32_MAX || nz > UINT32_MAX) return SZO_ERR_ARG;
    const size_t n = nx * ny * nz, pl = nx * ny;
    if (n && !x) return SZO_ERR_ARG;
    if (cap < SZO_LORENZO_HEAD) return SZO_ERR_CAP;
    const double inv = (double)(1.0f / eb);
    int32_t *q = (int32_t *)malloc(sizeof(int32_t) * (n ? n : 1));
    int32_t *r = (int32_t *)malloc(sizeof(int32_t) * (n ? n : 1));
    if (!q || !r) { free(q); free(r); return SZO_ERR_NOMEM; }
    for (size_t e = 0; e < n; e++) q[e] = q_at(x, KIND_FLOAT, e, inv);
    for (size_t e = 0; e < n; e++) {
        const size_t j = (e / nx) % ny, k = e / pl;
        uint32_t v = (uint32_t)q[e];
        if (j) v -= (uint32_t)q[e - nx];
        if (k) v -= (uint32_t)q[e - pl];
        if (j && k) v += (uint32_t)q[e - nx - pl];
        r[e] = (int32_t)v;
    }
    put_u32le(out, (uint32_t)nx);
    put_u32le(out + 4, (uint32_t)ny);
    put_u32le(out + 8, (uint32_t)nz);
    unsigned char ebb[4], be[4];
    memcpy(ebb, &eb, 4);
    be[0] = ebb[3]; be[1] = ebb[2]; be[2] = ebb[1]; be[3] = ebb[0];
    size_t sz = 0;
    int rc = compress_any(r, KIND_Q_F, n, 0.0, be, 32, T, 1, out + SZO_LORENZO_HEAD, cap - SZO_LORENZO_HEAD, &sz);
    if (rc == SZO_OK) *out_size = sz + SZO_LORENZO_HEAD;
    free(q);
    free(r);
    return rc;
}

int szo_lorenzo_decompress(const unsigned char *stream, size_t len, size_t nx, size_t ny, size_t nz, int T, float *y)
{
    const size_t n = nx * ny * nz, pl = nx * ny;
    if (!stream || T <= 0 || (n && !y)) return SZO_ERR_ARG;
    if (len < SZO_LORENZO_HEAD + 4) return SZO_ERR_STREAM;
    if (get_u32le(stream) != nx || get_u32le(stream + 4) != ny || get_u32le(stream + 8) != nz) return SZO_ERR_ARG;
    const unsigned char *s = stream + SZO_LORENZO_HEAD;
    int32_t *q = (int32_t *)malloc(sizeof(int32_t) * (n ? n : 1));
    if (!q) return SZO_ERR_NOMEM;
    int rc = decompress_any(s, len - SZO_LORENZO_HEAD, n, 32, T, 1, 0.0, KIND_Q_F, q);
    if (rc == SZO_OK) {
        unsigned char ebb[4] = {s[3], s[2], s[1], s[0]};
        float eb;
        memcpy(&eb, ebb, 4);
        for (size_t k = 0; k < nz; k++)  /* sums along y */
            for (size_t i = 0; i < nx; i++) {
                uint32_t run = 0;
                for (size_t j = 0; j < ny; j++) {
                    const size_t e = k * pl + j * nx + i;
                    run += (uint32_t)q[e];
                    q[e] = (int32_t)run;
                }
            }
        for (size_t j = 0; j < ny; j++)  /* sums along z */
            for (size_t i = 0; i < nx; i++) {
                uint32_t run = 0;
                for (size_t k = 0; k < nz; k++) {
                    const size_t e = k * pl + j * nx + i;
                    run += (uint32_t)q[e];
                    q[e] = (int32_t)run;
                }
            }
        for (size_t e = 0; e < n; e++) y[e] = dequant(q[e], eb);
    }
    free(q);
    return rc;
}
