/*
 * hd_oracle.c — CPU restatement of ssciwr/hammingdist 1.4.0's pairwise
 * Hamming-distance path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker: it is called by tests/,
 * by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, never by the
 * product path (hammingdist_gb300/, which runs on the GPU only).
 *
 * Parity pinning: every function below is checked against outputs of the
 * reference itself (built from its sources by oracle/build_ref.sh) through the
 * fixtures in tests/golden/, generated by tests/golden/make_golden.py.
 *
 * Each function cites the reference file:line whose behaviour it restates.
 * Plain C11 + OpenMP; no architecture intrinsics (it is built on x86_64 and on
 * aarch64).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define HDO_OK 0
#define HDO_ERR_EMPTY -1       /* "Error: Empty sequence" */
#define HDO_ERR_LENGTH -2      /* "Error: Sequences do not all have the same length" */
#define HDO_ERR_ALLOC -3
#define HDO_ERR_ARG -4
#define HDO_ERR_REF_SHORT -5   /* a sequence longer than the reference */

/* ------------------------------------------------------------------------ */
/* Encoding: src/hamming_impl.cc:23-44 (lookupTable). Two nibbles per byte
 * value; '-' = 0xff, A/C/G/T one-hot, X = 0x33 only when include_x, every other
 * byte 0. Bytes >= 0x80 are indexed unsigned here (the reference indexes with
 * a plain char, which is undefined for them on x86); they map to 0.          */
void hdo_lookup(int include_x, uint8_t table[256]) {
  memset(table, 0, 256);
  table['-'] = 0xff;
  table['A'] = 0x11;
  table['C'] = 0x22;
  table['G'] = 0x44;
  table['T'] = 0x88;
  if (include_x) table['X'] = 0x33;
}

/* ------------------------------------------------------------------------ */
/* std::getline over a byte buffer, with the stream's eof flag.              */
typedef struct {
  const char *buf;
  size_t n, pos;
  int eof;
} hdo_lines;

static int hdo_getline(hdo_lines *lr, size_t *start, size_t *len) {
  if (lr->pos >= lr->n) { /* nothing left: eofbit + failbit */
    lr->eof = 1;
    return 0;
  }
  const char *p = memchr(lr->buf + lr->pos, '\n', lr->n - lr->pos);
  *start = lr->pos;
  if (p) {
    *len = (size_t)(p - (lr->buf + lr->pos));
    lr->pos = (size_t)(p - lr->buf) + 1;
  } else { /* last line without '\n': extracted, eofbit set, success */
    *len = lr->n - lr->pos;
    lr->pos = lr->n;
    lr->eof = 1;
  }
  return 1;
}

/* A growable byte string. */
typedef struct {
  char *p;
  size_t n, cap;
} hdo_str;

static int hdo_str_append(hdo_str *s, const char *src, size_t len) {
  if (s->n + len > s->cap) {
    size_t cap = s->cap ? s->cap : 64;
    while (cap < s->n + len) cap *= 2;
    char *q = realloc(s->p, cap);
    if (!q) return HDO_ERR_ALLOC;
    s->p = q;
    s->cap = cap;
  }
  memcpy(s->p + s->n, src, len);
  s->n += len;
  return HDO_OK;
}

/* Parsed records: concatenated sequence bytes + n+1 offsets. */
typedef struct {
  hdo_str bytes;
  uint64_t *offsets; /* n + 1 entries */
  uint64_t n, cap;
} hdo_records;

static int hdo_records_push(hdo_records *r, const hdo_str *seq) {
  if (r->n + 2 > r->cap) {
    uint64_t cap = r->cap ? r->cap * 2 : 1024;
    uint64_t *q = realloc(r->offsets, cap * sizeof(uint64_t));
    if (!q) return HDO_ERR_ALLOC;
    r->offsets = q;
    r->cap = cap;
  }
  if (r->n == 0) r->offsets[0] = 0;
  if (hdo_str_append(&r->bytes, seq->p ? seq->p : "", seq->n)) return HDO_ERR_ALLOC;
  r->offsets[r->n + 1] = r->bytes.n;
  r->n++;
  return HDO_OK;
}

/* Record parser: src/hamming_impl.cc:211-233 (read_fasta without the map),
 * also the loops of src/hamming.cc:89-101 and :119-140. The first line is
 * skipped whatever it holds; a record is every line up to the next line whose
 * first byte is '>' (that header line is consumed); empty lines append
 * nothing; the loop stops after n_limit records (0 = no limit) or when the
 * stream has reached its end.                                                */
static int hdo_parse(const char *buf, size_t nbytes, uint64_t n_limit,
                     hdo_records *out) {
  hdo_lines lr = {buf, nbytes, 0, 0};
  size_t s, l;
  hdo_str seq = {0};
  memset(out, 0, sizeof(*out));
  if (n_limit == 0) n_limit = UINT64_MAX;
  hdo_getline(&lr, &s, &l); /* skip first header */
  uint64_t count = 0;
  while (count < n_limit && !lr.eof) {
    seq.n = 0;
    while (hdo_getline(&lr, &s, &l) && !(l > 0 && buf[s] == '>')) {
      if (hdo_str_append(&seq, buf + s, l)) return HDO_ERR_ALLOC;
    }
    if (hdo_records_push(out, &seq)) return HDO_ERR_ALLOC;
    ++count;
  }
  free(seq.p);
  if (out->n == 0) {
    out->offsets = calloc(1, sizeof(uint64_t));
  }
  return HDO_OK;
}

static uint64_t hdo_hash(const char *p, size_t n) {
  uint64_t h = 1469598103934665603ull; /* FNV-1a */
  for (size_t i = 0; i < n; ++i) {
    h ^= (uint8_t)p[i];
    h *= 1099511628211ull;
  }
  return h ^ (n * 0x9e3779b97f4a7c15ull);
}

/* Duplicate removal: src/hamming_impl.cc:223-240. Unique rows are numbered in
 * order of first occurrence; index[k] is the unique row of input record k.
 * Equality is on the raw bytes of the record.                                */
static int hdo_dedupe(const hdo_records *in, hdo_records *uniq, uint64_t *index) {
  uint64_t cap = 16;
  while (cap < 2 * in->n + 2) cap *= 2;
  int64_t *table = malloc(cap * sizeof(int64_t));
  if (!table) return HDO_ERR_ALLOC;
  for (uint64_t i = 0; i < cap; ++i) table[i] = -1;
  uint64_t *first = malloc((in->n + 1) * sizeof(uint64_t)); /* unique -> record */
  if (!first) return HDO_ERR_ALLOC;
  uint64_t n_unique = 0;
  for (uint64_t k = 0; k < in->n; ++k) {
    const char *p = in->bytes.p + in->offsets[k];
    size_t len = in->offsets[k + 1] - in->offsets[k];
    uint64_t slot = hdo_hash(p, len) & (cap - 1);
    for (;;) {
      int64_t u = table[slot];
      if (u < 0) {
        table[slot] = (int64_t)n_unique;
        first[n_unique] = k;
        index[k] = n_unique++;
        break;
      }
      uint64_t r = first[u];
      size_t rl = in->offsets[r + 1] - in->offsets[r];
      if (rl == len && memcmp(in->bytes.p + in->offsets[r], p, len) == 0) {
        index[k] = (uint64_t)u;
        break;
      }
      slot = (slot + 1) & (cap - 1);
    }
  }
  memset(uniq, 0, sizeof(*uniq));
  for (uint64_t u = 0; u < n_unique; ++u) {
    uint64_t r = first[u];
    hdo_str tmp = {in->bytes.p + in->offsets[r], in->offsets[r + 1] - in->offsets[r], 0};
    if (hdo_records_push(uniq, &tmp)) return HDO_ERR_ALLOC;
  }
  if (uniq->n == 0) uniq->offsets = calloc(1, sizeof(uint64_t));
  free(table);
  free(first);
  return HDO_OK;
}

static void hdo_records_free(hdo_records *r) {
  free(r->bytes.p);
  free(r->offsets);
  memset(r, 0, sizeof(*r));
}

/* validate_data: src/hamming_impl.cc:80-91. */
static int hdo_validate(const hdo_records *r) {
  if (r->n == 0 || r->offsets[1] == r->offsets[0]) return HDO_ERR_EMPTY;
  uint64_t len = r->offsets[1] - r->offsets[0];
  for (uint64_t k = 0; k < r->n; ++k)
    if (r->offsets[k + 1] - r->offsets[k] != len) return HDO_ERR_LENGTH;
  return HDO_OK;
}

/* ------------------------------------------------------------------------ */
/* from_string: src/hamming_impl.cc:244-267. Site 2k in the low nibble, 2k+1 in
 * the high nibble, always with lookupTable(false); an odd tail gets a '-'
 * high nibble; the row is padded with 0xff bytes to a multiple of 8.         */
uint64_t hdo_packed_row_bytes(uint64_t L) { return ((L + 1) / 2 + 7) / 8 * 8; }

void hdo_pack_row(const char *seq, uint64_t L, uint8_t *out) {
  uint8_t lk[256];
  hdo_lookup(0, lk);
  uint64_t nb = hdo_packed_row_bytes(L);
  uint64_t k = 0;
  for (; 2 * k + 1 < L; ++k)
    out[k] = (uint8_t)((lk[(uint8_t)seq[2 * k]] & 0x0f) | (lk[(uint8_t)seq[2 * k + 1]] & 0xf0));
  if (2 * k < L) {
    out[k] = (uint8_t)((lk[(uint8_t)seq[2 * k]] & 0x0f) | 0xf0);
    ++k;
  }
  for (; k < nb; ++k) out[k] = 0xff;
}

/* Dense AND rule: distance_cpp, src/hamming_impl.cc:131-140, in the form of
 * the reference's SIMD kernels (src/distance_neon.cc:6-69; the SSE2/AVX2/
 * AVX-512 files are the same algorithm at other widths): per 16-byte vector,
 * c = a & b; each nibble of c that is zero adds 1 to a uint8 lane counter;
 * lanes are summed after at most 127 vectors (16 when max_dist < 255) and the
 * count returns early once it reaches max_dist. GCC generic vectors make this
 * NEON on aarch64 and SSE2 on x86_64 without architecture intrinsics.      */
typedef uint8_t hdo_v16u8 __attribute__((vector_size(16)));

static int hdo_distance_dense(const uint8_t *a, const uint8_t *b, uint64_t nbytes,
                              int max_dist) {
  const hdo_v16u8 zero = {0};
  const hdo_v16u8 m0 = zero + 0x0f, m1 = zero + 0xf0;
  int r = 0;
  const uint64_t n_iter = nbytes / 16;
  const uint64_t n_inner = max_dist >= 255 ? 127 : 16;
  for (uint64_t i0 = 0; i0 < n_iter; i0 += n_inner) {
    const uint64_t i1 = i0 + n_inner < n_iter ? i0 + n_inner : n_iter;
    hdo_v16u8 acc = zero;
    for (uint64_t i = i0; i < i1; ++i) {
      hdo_v16u8 x, y;
      memcpy(&x, a + 16 * i, 16);
      memcpy(&y, b + 16 * i, 16);
      const hdo_v16u8 c = x & y;
      acc -= (hdo_v16u8)((c & m0) == zero);  /* -1 per zero nibble */
      acc -= (hdo_v16u8)((c & m1) == zero);
    }
    int blk = 0;
    for (int k = 0; k < 16; ++k) blk += acc[k];
    r += blk;
    if (r >= max_dist) return max_dist;
  }
  for (uint64_t i = n_iter * 16; i < nbytes; ++i) {
    uint8_t c = a[i] & b[i];
    r += ((c & 0x0f) == 0) + ((c & 0xf0) == 0);
  }
  return r < max_dist ? r : max_dist;
}

/* safe_int_cast: include/hamming/hamming_impl.hh:37-45 — values above the
 * type's maximum saturate; negative ints wrap through static_cast.          */
static uint32_t hdo_clamp_max(int64_t max_distance, int dtype_bytes) {
  uint32_t tmax = dtype_bytes == 1 ? 0xffu : 0xffffu;
  if (max_distance > (int64_t)tmax) return tmax;
  return (uint32_t)((uint64_t)max_distance & tmax);
}

/* Dense lower triangle: the OpenMP loop of include/hamming/hamming_impl.hh:
 * 161-175. lt[i(i-1)/2 + j] for i > j.                                      */
int hdo_lt_dense(const uint8_t *packed, uint64_t n, uint64_t row_bytes,
                 int64_t max_distance, int dtype_bytes, void *out) {
  if (dtype_bytes != 1 && dtype_bytes != 2 && dtype_bytes != 4) return HDO_ERR_ARG;
  int max_dist = dtype_bytes == 4 ? (int)max_distance
                                  : (int)hdo_clamp_max(max_distance, dtype_bytes);
#pragma omp parallel for schedule(static, 1)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    uint64_t off = (uint64_t)i * (uint64_t)(i - 1) / 2;
    for (int64_t j = 0; j < i; ++j) {
      int d = hdo_distance_dense(packed + (uint64_t)i * row_bytes,
                                 packed + (uint64_t)j * row_bytes, row_bytes, max_dist);
      if (dtype_bytes == 1) ((uint8_t *)out)[off + j] = (uint8_t)d;
      else if (dtype_bytes == 2) ((uint16_t *)out)[off + j] = (uint16_t)d;
      else ((uint32_t *)out)[off + j] = (uint32_t)d;
    }
  }
  return HDO_OK;
}

/* ------------------------------------------------------------------------ */
/* Consensus: get_reference_expression, src/hamming_impl.cc:142-168. Per site
 * the most frequent of A, C, G, T (and X with include_x); ties go to the first
 * in that order; a site with none of them gets 'A'.                         */
static void hdo_consensus(const hdo_records *r, uint64_t L, int include_x, char *g0) {
  static const char itoc[6] = {'A', 'A', 'C', 'G', 'T', 'X'};
  uint8_t ctoi[256];
  memset(ctoi, 0, sizeof(ctoi));
  ctoi['A'] = 1; ctoi['C'] = 2; ctoi['G'] = 3; ctoi['T'] = 4;
  if (include_x) ctoi['X'] = 5;
#pragma omp parallel for
  for (int64_t s = 0; s < (int64_t)L; ++s) {
    uint64_t cnt[6] = {0, 0, 0, 0, 0, 0};
    for (uint64_t k = 0; k < r->n; ++k)
      ++cnt[ctoi[(uint8_t)r->bytes.p[r->offsets[k] + s]]];
    int best = 1;
    for (int c = 2; c < 6; ++c)
      if (cnt[c] > cnt[best]) best = c;
    g0[s] = itoc[best];
  }
}

/* Sparse form: to_sparse_data, src/hamming_impl.cc:170-188 — per sequence the
 * list of (site, code) where the byte differs from the consensus byte.       */
typedef struct {
  uint64_t *site;
  uint8_t *code;
  uint64_t n;
} hdo_sparse;

/* distance_sparse: src/hamming_impl.cc:93-129 (merge of two sorted lists). */
static int hdo_distance_sparse(const hdo_sparse *a, const hdo_sparse *b, int max_dist) {
  int r = 0;
  uint64_t ia = 0, ib = 0;
  while (ia < a->n && ib < b->n) {
    if (a->site[ia] < b->site[ib]) {
      r += a->code[ia] != 0xff;
      ++ia;
    } else if (a->site[ia] > b->site[ib]) {
      r += b->code[ib] != 0xff;
      ++ib;
    } else {
      int nodash = a->code[ia] != 0xff && b->code[ib] != 0xff;
      r += nodash && a->code[ia] != b->code[ib];
      ++ia;
      ++ib;
    }
    if (r >= max_dist) return max_dist;
  }
  for (; ia < a->n; ++ia) r += a->code[ia] != 0xff;
  for (; ib < b->n; ++ib) r += b->code[ib] != 0xff;
  return r < max_dist ? r : max_dist;
}

/* distances<T> with use_gpu=False: include/hamming/hamming_impl.hh:68-176.
 * include_x forces the sparse rule; otherwise the sparse rule is taken when
 * fewer than 0.5% of all sites differ from the consensus (:104-118), else the
 * dense AND rule. *used_sparse reports the branch (the reference prints it). */
int hdo_lt_cpu(const char *seqs, const uint64_t *offsets, uint64_t n, int include_x,
               int64_t max_distance, int dtype_bytes, void *out, int *used_sparse) {
  if (dtype_bytes != 1 && dtype_bytes != 2) return HDO_ERR_ARG;
  hdo_records r = {{(char *)seqs, offsets[n], 0}, (uint64_t *)offsets, n, 0};
  int rc = hdo_validate(&r);
  if (rc) return rc;
  uint64_t L = offsets[1] - offsets[0];
  int max_dist = (int)hdo_clamp_max(max_distance, dtype_bytes);
  char *g0 = malloc(L);
  uint8_t lk[256];
  hdo_lookup(include_x, lk);
  hdo_consensus(&r, L, include_x, g0);
  hdo_sparse *sp = calloc(n, sizeof(hdo_sparse));
  uint64_t n_diff = 0;
  for (uint64_t k = 0; k < n; ++k) {
    const char *s = seqs + offsets[k];
    uint64_t m = 0;
    for (uint64_t i = 0; i < L; ++i) m += s[i] != g0[i];
    sp[k].site = malloc((m + 1) * sizeof(uint64_t));
    sp[k].code = malloc(m + 1);
    for (uint64_t i = 0; i < L; ++i)
      if (s[i] != g0[i]) {
        sp[k].site[sp[k].n] = i;
        sp[k].code[sp[k].n++] = lk[(uint8_t)s[i]];
      }
    n_diff += m;
  }
  int use_sparse = include_x;
  if (!include_x) {
    double frac = (double)n_diff / (double)(n * L);
    use_sparse = frac < 0.005;
  }
  *used_sparse = use_sparse;
  if (use_sparse) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      uint64_t off = (uint64_t)i * (uint64_t)(i - 1) / 2;
      for (int64_t j = 0; j < i; ++j) {
        int d = hdo_distance_sparse(&sp[i], &sp[j], max_dist);
        if (dtype_bytes == 1) ((uint8_t *)out)[off + j] = (uint8_t)d;
        else ((uint16_t *)out)[off + j] = (uint16_t)d;
      }
    }
  } else {
    uint64_t rb = hdo_packed_row_bytes(L);
    uint8_t *packed = malloc(n * rb);
    for (uint64_t k = 0; k < n; ++k) hdo_pack_row(seqs + offsets[k], L, packed + k * rb);
    hdo_lt_dense(packed, n, rb, max_distance, dtype_bytes, out);
    free(packed);
  }
  for (uint64_t k = 0; k < n; ++k) {
    free(sp[k].site);
    free(sp[k].code);
  }
  free(sp);
  free(g0);
  return HDO_OK;
}

/* ------------------------------------------------------------------------ */
/* Reference-distance rule: distance(), src/hamming.cc:54-74 — a site counts
 * when the codes share no bit, or when the bytes differ and neither is '-'. */
static inline uint32_t hdo_ref_site(uint8_t ca, uint8_t cb, const uint8_t *lk) {
  uint8_t a = lk[ca], b = lk[cb];
  int invalid = (a & b) == 0;
  int differ = ca != cb;
  int nodash = a != 0xff && b != 0xff;
  return (uint32_t)(invalid || (differ && nodash));
}

int hdo_distance(const char *s0, uint64_t l0, const char *s1, uint64_t l1,
                 int include_x, uint32_t *out) {
  if (l0 != l1) return HDO_ERR_LENGTH;
  uint8_t lk[256];
  hdo_lookup(include_x, lk);
  uint32_t d = 0;
  for (uint64_t i = 0; i < l0; ++i) d += hdo_ref_site((uint8_t)s0[i], (uint8_t)s1[i], lk);
  *out = d;
  return HDO_OK;
}

/* ------------------------------------------------------------------------ */
/* Entry points over a FASTA byte buffer.                                    */

/* Parse (+ optional dedupe): read_fasta, src/hamming_impl.cc:200-242.
 * Returns malloc'd concatenated sequences + offsets (n+1) and, with
 * remove_duplicates, the per-input indices (n_input entries).               */
int hdo_read_fasta(const char *buf, size_t nbytes, int remove_duplicates, uint64_t n_limit,
                   char **seqs, uint64_t **offsets, uint64_t *n,
                   uint64_t **indices, uint64_t *n_input) {
  hdo_records rec;
  int rc = hdo_parse(buf, nbytes, n_limit, &rec);
  if (rc) return rc;
  *n_input = rec.n;
  *indices = NULL;
  if (remove_duplicates) {
    uint64_t *idx = malloc((rec.n + 1) * sizeof(uint64_t));
    hdo_records u;
    rc = hdo_dedupe(&rec, &u, idx);
    if (rc) return rc;
    hdo_records_free(&rec);
    rec = u;
    *indices = idx;
  }
  *seqs = rec.bytes.p;
  *offsets = rec.offsets;
  *n = rec.n;
  return HDO_OK;
}

/* fasta_sequence_indices: src/hamming.cc:76-102 (always deduplicates). */
int hdo_fasta_sequence_indices(const char *buf, size_t nbytes, uint64_t n_limit,
                               uint64_t **indices, uint64_t *n_input) {
  char *seqs;
  uint64_t *offsets, n;
  int rc = hdo_read_fasta(buf, nbytes, 1, n_limit, &seqs, &offsets, &n, indices, n_input);
  free(seqs);
  free(offsets);
  return rc;
}

/* fasta_reference_distances: src/hamming.cc:104-141. One distance per record
 * (no n limit, no dedupe). The reference does not check lengths; a record
 * longer than the reference is reported as HDO_ERR_REF_SHORT here (the
 * reference reads past its buffer in that case).                           */
int hdo_reference_distances(const char *ref, uint64_t ref_len, const char *buf,
                            size_t nbytes, int include_x, uint32_t **out, uint64_t *n_out) {
  hdo_records rec;
  int rc = hdo_parse(buf, nbytes, 0, &rec);
  if (rc) return rc;
  uint8_t lk[256];
  hdo_lookup(include_x, lk);
  uint32_t *d = malloc((rec.n + 1) * sizeof(uint32_t));
  for (uint64_t k = 0; k < rec.n; ++k) {
    uint64_t len = rec.offsets[k + 1] - rec.offsets[k];
    if (len > ref_len) {
      free(d);
      hdo_records_free(&rec);
      return HDO_ERR_REF_SHORT;
    }
  }
#pragma omp parallel for
  for (int64_t k = 0; k < (int64_t)rec.n; ++k) {
    const char *s = rec.bytes.p + rec.offsets[k];
    uint64_t len = rec.offsets[k + 1] - rec.offsets[k];
    uint32_t acc = 0;
    for (uint64_t i = 0; i < len; ++i) acc += hdo_ref_site((uint8_t)s[i], (uint8_t)ref[i], lk);
    d[k] = acc;
  }
  *out = d;
  *n_out = rec.n;
  hdo_records_free(&rec);
  return HDO_OK;
}

/* from_fasta(use_gpu=True) semantics end to end on the CPU: read_fasta +
 * validate_data + to_dense_data + the dense loop (the reference GPU kernel,
 * src/distance_cuda.cu:9-89, applies the same AND rule). out must hold
 * n_unique(n_unique-1)/2 entries; pass out=NULL to query *n_rows first.    */
int hdo_from_fasta_dense(const char *buf, size_t nbytes, int remove_duplicates,
                         uint64_t n_limit, int64_t max_distance, int dtype_bytes,
                         void *out, uint64_t out_capacity, uint64_t *n_rows,
                         uint64_t *indices_out, uint64_t *n_input) {
  char *seqs;
  uint64_t *offsets, n, *idx;
  int rc = hdo_read_fasta(buf, nbytes, remove_duplicates, n_limit, &seqs, &offsets, &n,
                          &idx, n_input);
  if (rc) return rc;
  hdo_records r = {{seqs, offsets[n], 0}, offsets, n, 0};
  rc = hdo_validate(&r);
  *n_rows = n;
  if (!rc && out) {
    if (out_capacity < n * (n - 1) / 2) {
      rc = HDO_ERR_ARG;
    } else {
      uint64_t L = offsets[1] - offsets[0];
      uint64_t rb = hdo_packed_row_bytes(L);
      uint8_t *packed = malloc(n * rb);
#pragma omp parallel for
      for (int64_t k = 0; k < (int64_t)n; ++k)
        hdo_pack_row(seqs + offsets[k], L, packed + (uint64_t)k * rb);
      rc = hdo_lt_dense(packed, n, rb, max_distance, dtype_bytes, out);
      free(packed);
    }
  }
  if (indices_out && idx) memcpy(indices_out, idx, *n_input * sizeof(uint64_t));
  free(seqs);
  free(offsets);
  free(idx);
  return rc;
}

/* The same in one pass over the text, as the reference's from_fasta reads
 * its file once (include/hamming/hamming.hh:168-178): the lower triangle is
 * returned in *out (malloc'd, n(n-1)/2 entries of dtype_bytes, release with
 * hdo_free) and, with remove_duplicates, the sequence indices in *indices.  */
int hdo_from_fasta_dense_once(const char *buf, size_t nbytes, int remove_duplicates,
                              uint64_t n_limit, int64_t max_distance, int dtype_bytes,
                              void **out, uint64_t *n_rows, uint64_t **indices,
                              uint64_t *n_input) {
  char *seqs;
  uint64_t *offsets, n, *idx;
  *out = NULL;
  *indices = NULL;
  if (dtype_bytes != 1 && dtype_bytes != 2 && dtype_bytes != 4) return HDO_ERR_ARG;
  int rc = hdo_read_fasta(buf, nbytes, remove_duplicates, n_limit, &seqs, &offsets, &n,
                          &idx, n_input);
  if (rc) return rc;
  hdo_records r = {{seqs, offsets[n], 0}, offsets, n, 0};
  rc = hdo_validate(&r);
  *n_rows = n;
  if (!rc) {
    const uint64_t entries = n * (n - 1) / 2;
    uint64_t L = offsets[1] - offsets[0];
    uint64_t rb = hdo_packed_row_bytes(L);
    uint8_t *packed = malloc(n * rb);
    void *lt = malloc((entries ? entries : 1) * (uint64_t)dtype_bytes);
    if (!packed || !lt) {
      free(packed);
      free(lt);
      rc = HDO_ERR_ALLOC;
    } else {
#pragma omp parallel for
      for (int64_t k = 0; k < (int64_t)n; ++k)
        hdo_pack_row(seqs + offsets[k], L, packed + (uint64_t)k * rb);
      rc = hdo_lt_dense(packed, n, rb, max_distance, dtype_bytes, lt);
      free(packed);
      if (rc) free(lt);
      else *out = lt;
    }
  }
  if (!rc) *indices = idx;
  else free(idx);
  free(seqs);
  free(offsets);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* Writers.                                                                  */

static size_t hdo_utoa(uint64_t v, char *dst) {
  char tmp[24];
  size_t n = 0;
  do {
    tmp[n++] = (char)('0' + v % 10);
    v /= 10;
  } while (v);
  for (size_t i = 0; i < n; ++i) dst[i] = tmp[n - 1 - i];
  return n;
}

static uint64_t hdo_lt_get(const void *lt, int dtype_bytes, uint64_t k) {
  if (dtype_bytes == 1) return ((const uint8_t *)lt)[k];
  if (dtype_bytes == 2) return ((const uint16_t *)lt)[k];
  return ((const uint32_t *)lt)[k];
}

/* Lower-triangular text: lower_triangular_lines / partial_write_lower_
 * triangular, include/hamming/hamming_utils.hh:19-110. Row i = 1..n-1 is
 * "d(i,0),...,d(i,i-1)\n". Writes into dst (NULL = size query); returns the
 * number of bytes.                                                          */
uint64_t hdo_format_lower_triangular(const void *lt, uint64_t n_entries, int dtype_bytes,
                                     char *dst) {
  uint64_t pos = 0, k = 0;
  char tmp[24];
  for (uint64_t i = 1; k < n_entries; ++i) {
    for (uint64_t j = 0; j < i && k < n_entries; ++j, ++k) {
      size_t m = hdo_utoa(hdo_lt_get(lt, dtype_bytes, k), tmp);
      if (dst) memcpy(dst + pos, tmp, m);
      pos += m;
      if (dst) dst[pos] = (j + 1 == i) ? '\n' : ',';
      pos += 1;
    }
  }
  return pos;
}

/* Sparse text: DataSet::dump_sparse, include/hamming/hamming.hh:79-114 —
 * "i j d\n" for every i > j with d <= threshold, rows in ascending order (the
 * serial order of the reference; its OpenMP build may emit 200-row blocks in
 * any order). Returns bytes; dst NULL = size query.                        */
uint64_t hdo_format_sparse(const void *lt, uint64_t nsamples, int dtype_bytes,
                           int64_t threshold, char *dst, uint64_t *n_lines) {
  uint64_t pos = 0, k = 0, lines = 0;
  char tmp[72];
  for (uint64_t i = 1; i < nsamples; ++i) {
    for (uint64_t j = 0; j < i; ++j, ++k) {
      uint64_t d = hdo_lt_get(lt, dtype_bytes, k);
      if ((int64_t)d <= threshold) {
        size_t m = hdo_utoa(i, tmp);
        tmp[m++] = ' ';
        m += hdo_utoa(j, tmp + m);
        tmp[m++] = ' ';
        m += hdo_utoa(d, tmp + m);
        tmp[m++] = '\n';
        if (dst) memcpy(dst + pos, tmp, m);
        pos += m;
        ++lines;
      }
    }
  }
  if (n_lines) *n_lines = lines;
  return pos;
}

void hdo_free(void *p) { free(p); }

int hdo_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------ result file formats
 * Single-threaded, like the reference's host code. */

/* DataSet::dump (include/hamming/hamming.hh:63-73): the full matrix, entries
 * (*this)[{i, j}] (129-138: 0 on the diagonal, symmetric), ", " between
 * entries, one line per row; an index past `entries` reads as 0. */
int hdo_dump_full(const void *lt, uint64_t entries, uint64_t n, int dtype_bytes, const char *path) {
  FILE *f = fopen(path, "wb");
  if (!f) return -5;
  char *line = (char *)malloc(n * 12 + 2);
  if (!line && n) {
    fclose(f);
    return -10;
  }
  for (uint64_t i = 0; i < n; ++i) {
    size_t m = 0;
    for (uint64_t j = 0; j < n; ++j) {
      uint64_t v = 0;
      if (i != j) {
        const uint64_t k = i > j ? i * (i - 1) / 2 + j : j * (j - 1) / 2 + i;
        v = k < entries ? hdo_lt_get(lt, dtype_bytes, k) : 0;
      }
      m += hdo_utoa(v, line + m);
      if (j != n - 1) {
        line[m++] = ',';
        line[m++] = ' ';
      }
    }
    line[m++] = '\n';
    if (fwrite(line, 1, m, f) != m) {
      free(line);
      fclose(f);
      return -5;
    }
  }
  free(line);
  return fclose(f) == 0 ? 0 : -5;
}

/* std::stoi on [p, end): C whitespace, sign, digits; 0 ok, 1 no digits
 * (std::invalid_argument), 2 outside int (std::out_of_range). */
static int hdo_stoi(const char *p, const char *end, int *v) {
  while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\v' || *p == '\f' || *p == '\r'))
    ++p;
  int neg = 0;
  if (p < end && (*p == '+' || *p == '-')) neg = *p++ == '-';
  const char *d0 = p;
  long long acc = 0;
  while (p < end && *p >= '0' && *p <= '9') {
    if (acc < (1ll << 40)) acc = acc * 10 + (*p - '0');
    ++p;
  }
  if (p == d0) return 1;
  if (neg) acc = -acc;
  if (acc > 2147483647ll || acc < -2147483648ll) return 2;
  *v = (int)acc;
  return 0;
}

static char *hdo_slurp(const char *path, uint64_t *n) {
  FILE *f = fopen(path, "rb");
  if (!f) return NULL;
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  char *buf = (char *)malloc((size_t)sz + 1);
  if (buf && sz > 0 && fread(buf, 1, (size_t)sz, f) != (size_t)sz) {
    free(buf);
    buf = NULL;
  }
  fclose(f);
  *n = (uint64_t)sz;
  return buf;
}

/* from_lower_triangular<T> (hamming.hh:152-166): every comma-separated field
 * of every line (std::getline while the stream is good), safe_int_cast<T>
 * (include/hamming/hamming_impl.hh:37-45); nsamples = (round(sqrt(8 size +
 * 1)) + 1) / 2. *out from malloc. */
int hdo_read_lower_triangular(const char *path, int dtype_bytes, void **out, uint64_t *entries,
                              uint64_t *nsamples, int *parse_error) {
  uint64_t n = 0;
  *parse_error = 0;
  char *buf = hdo_slurp(path, &n);
  if (!buf) return -5;
  uint64_t cap = 1024, cnt = 0;
  uint8_t *vals = (uint8_t *)malloc(cap * dtype_bytes);
  const int mx = dtype_bytes == 1 ? 255 : 65535;
  uint64_t s = 0;
  while (s < n) {  /* one line [s, e) */
    uint64_t e = s;
    while (e < n && buf[e] != '\n') ++e;
    uint64_t a = s;
    for (;;) {  /* field [a, b) */
      uint64_t b = a;
      while (b < e && buf[b] != ',') ++b;
      int v = 0;
      const int r = hdo_stoi(buf + a, buf + e, &v);
      if (r) {
        *parse_error = r;
        free(vals);
        free(buf);
        return -12;
      }
      if (cnt == cap) {
        cap *= 2;
        vals = (uint8_t *)realloc(vals, cap * dtype_bytes);
      }
      const unsigned u = v > mx ? (unsigned)mx : (unsigned)v;
      if (dtype_bytes == 1) vals[cnt] = (uint8_t)u;
      else ((uint16_t *)vals)[cnt] = (uint16_t)u;
      ++cnt;
      if (b >= e) break;
      a = b + 1;
    }
    s = e + 1;
  }
  free(buf);
  *out = vals;
  *entries = cnt;
  *nsamples = ((uint64_t)llround(sqrt((double)(8 * cnt + 1))) + 1) / 2;
  return 0;
}

/* from_csv / DataSet(filename) (hamming.hh:34-55): nsamples = number of
 * '\n', n(n+1)/2 zeroed values; line i gives its first i fields (missing
 * ones repeat the last field, as std::getline leaves it), std::stoi
 * truncated to uint8. */
int hdo_read_csv(const char *path, uint8_t **out, uint64_t *entries, uint64_t *nsamples,
                 int *parse_error) {
  uint64_t n = 0;
  *parse_error = 0;
  char *buf = hdo_slurp(path, &n);
  if (!buf) return -5;
  uint64_t nl = 0;
  for (uint64_t k = 0; k < n; ++k) nl += buf[k] == '\n';
  const uint64_t total = nl * (nl + 1) / 2;
  uint8_t *vals = (uint8_t *)calloc(total ? total : 1, 1);
  uint64_t s = 0, line = 0, pos = 0;
  while (s < n) {
    uint64_t e = s;
    while (e < n && buf[e] != '\n') ++e;
    uint64_t a = s;
    for (uint64_t j = 0; j < line; ++j) {
      int v = 0;
      const int r = hdo_stoi(buf + a, buf + e, &v);
      if (r) {
        *parse_error = r;
        free(vals);
        free(buf);
        return -12;
      }
      vals[pos++] = (uint8_t)(unsigned)v;
      uint64_t b = a;
      while (b < e && buf[b] != ',') ++b;
      if (b < e) a = b + 1;  /* else the line is exhausted: the same field again */
    }
    ++line;
    s = e + 1;
  }
  free(buf);
  *out = vals;
  *entries = total;
  *nsamples = nl;
  return 0;
}
