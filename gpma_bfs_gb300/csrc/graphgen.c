/*
 * graphgen.c - seeded synthetic edge streams and the reference's text format.
 *
 * The reference's demo reads a text file "n m" followed by m "src dst" lines
 * (gpma_bfs_demo.cu:6-30, dataset/prepare_dataset.sh:23-37: de-duplicated,
 * shuffled, 0-based). Its public dataset is not available offline, so these
 * generators produce edge lists of the same shape: R-MAT and Chung-Lu graphs
 * with self-loops and duplicate edges removed, then uniformly shuffled. All
 * randomness comes from xoshiro256** seeded through splitmix64; generation is
 * chunked with one stream per fixed-size chunk, so results do not depend on
 * the number of threads or on the host architecture.
 */
#include "../../include/gpma_gb300.h"

#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define GEN_CHUNK (1u << 20)

static uint64_t splitmix64(uint64_t *s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

typedef struct {
    uint64_t s[4];
} xoshiro;

static void xo_seed(xoshiro *x, uint64_t seed, uint64_t stream) {
    uint64_t sm = seed ^ (stream * 0xD1B54A32D192ED03ull);
    for (int i = 0; i < 4; ++i)
        x->s[i] = splitmix64(&sm);
}

static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t xo_next(xoshiro *x) {
    uint64_t *s = x->s;
    uint64_t result = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return result;
}

/* uniform integer in [0, bound) by 128-bit multiply (Lemire, no rejection:
 * bias < bound / 2^64, irrelevant at these sizes) */
static inline uint64_t xo_below(xoshiro *x, uint64_t bound) {
    return (uint64_t)(((unsigned __int128)xo_next(x) * bound) >> 64);
}

/* uniform double in [0, 1) with 53 random bits */
static inline double xo_unit(xoshiro *x) { return (double)(xo_next(x) >> 11) * (1.0 / 9007199254740992.0); }

/* LSD radix sort of u64, 11-bit digits, constant digits skipped. */
static int sort_u64(uint64_t *a, uint64_t n) {
    if (n < 2)
        return 0;
    uint64_t *tmp = (uint64_t *)malloc(n * sizeof(uint64_t));
    if (!tmp)
        return -1;
    uint64_t *src = a, *dst = tmp;
    static const int BITS = 11, BINS = 1 << 11;
    uint64_t *cnt = (uint64_t *)malloc(sizeof(uint64_t) * BINS);
    if (!cnt) {
        free(tmp);
        return -1;
    }
    for (int shift = 0; shift < 64; shift += BITS) {
        memset(cnt, 0, sizeof(uint64_t) * BINS);
        for (uint64_t i = 0; i < n; ++i)
            cnt[(src[i] >> shift) & (BINS - 1)]++;
        int trivial = 0;
        for (int d = 0; d < BINS; ++d)
            if (cnt[d] == n)
                trivial = 1;
        if (trivial)
            continue;
        uint64_t sum = 0;
        for (int d = 0; d < BINS; ++d) {
            uint64_t c = cnt[d];
            cnt[d] = sum;
            sum += c;
        }
        for (uint64_t i = 0; i < n; ++i)
            dst[cnt[(src[i] >> shift) & (BINS - 1)]++] = src[i];
        uint64_t *t = src;
        src = dst;
        dst = t;
    }
    if (src != a)
        memcpy(a, src, n * sizeof(uint64_t));
    free(cnt);
    free(tmp);
    return 0;
}

/* sort, drop duplicates and self-loops in place; returns the new count */
static uint64_t unique_no_loops(uint64_t *keys, uint64_t n) {
    sort_u64(keys, n);
    uint64_t w = 0;
    for (uint64_t i = 0; i < n; ++i) {
        uint64_t k = keys[i];
        if ((uint32_t)(k >> 32) == (uint32_t)k)
            continue;
        if (w > 0 && keys[w - 1] == k)
            continue;
        keys[w++] = k;
    }
    return w;
}

static void shuffle_u64(uint64_t *a, uint64_t n, uint64_t seed) {
    xoshiro x;
    xo_seed(&x, seed, 0xF15E5ull);
    for (uint64_t i = n; i > 1; --i) {
        uint64_t j = xo_below(&x, i);
        uint64_t t = a[i - 1];
        a[i - 1] = a[j];
        a[j] = t;
    }
}

static void split_keys(const uint64_t *keys, uint64_t m, uint32_t *src, uint32_t *dst) {
    for (uint64_t i = 0; i < m; ++i) {
        src[i] = (uint32_t)(keys[i] >> 32);
        dst[i] = (uint32_t)keys[i];
    }
}

gpma_status gpma_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                          uint32_t *src, uint32_t *dst, uint64_t capacity, uint64_t *m_out) {
    if (!src || !dst || !m_out || scale == 0 || scale > 31 || edge_factor == 0)
        return GPMA_ERR_INVALID;
    if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
        return GPMA_ERR_INVALID;
    uint64_t samples = (uint64_t)edge_factor << scale;
    if (capacity < samples)
        return GPMA_ERR_INVALID;
    uint64_t *keys = (uint64_t *)malloc(samples * sizeof(uint64_t));
    if (!keys)
        return GPMA_ERR_NOMEM;
    /* integer thresholds on 53-bit uniforms: quadrant (0,0) < ta <= (0,1) <
     * tab <= (1,0) < tabc <= (1,1) */
    const double two53 = 9007199254740992.0;
    uint64_t ta = (uint64_t)(a * two53), tab = (uint64_t)((a + b) * two53), tabc = (uint64_t)((a + b + c) * two53);
    uint64_t chunks = (samples + GEN_CHUNK - 1) / GEN_CHUNK;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t ch = 0; ch < (int64_t)chunks; ++ch) {
        xoshiro x;
        xo_seed(&x, seed, (uint64_t)ch + 1);
        uint64_t lo = (uint64_t)ch * GEN_CHUNK, hi = lo + GEN_CHUNK < samples ? lo + GEN_CHUNK : samples;
        for (uint64_t i = lo; i < hi; ++i) {
            uint32_t s = 0, d = 0;
            for (uint32_t lvl = 0; lvl < scale; ++lvl) {
                uint64_t r = xo_next(&x) >> 11;
                uint32_t sb = r >= tab, db = (r >= ta && r < tab) || r >= tabc;
                s = (s << 1) | sb;
                d = (d << 1) | db;
            }
            keys[i] = ((uint64_t)s << 32) | d;
        }
    }
    uint64_t m = unique_no_loops(keys, samples);
    shuffle_u64(keys, m, seed);
    split_keys(keys, m, src, dst);
    free(keys);
    *m_out = m;
    return GPMA_OK;
}

/* upper_bound over an increasing cumulative weight array */
static inline uint32_t pick(const double *cdf, uint32_t n, double u) {
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        uint32_t mid = lo + (hi - lo) / 2;
        if (cdf[mid] > u)
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo;
}

gpma_status gpma_gen_chung_lu(uint32_t n, uint64_t m, double exponent, uint32_t max_degree, uint64_t seed,
                              uint32_t *src, uint32_t *dst) {
    if (!src || !dst || n < 2 || m == 0 || exponent <= 1.0 || max_degree == 0)
        return GPMA_ERR_INVALID;
    if (m > (uint64_t)n * (n - 1) / 4)
        return GPMA_ERR_INVALID;
    /* expected degrees w_i = (i + i0)^-alpha, alpha = 1/(exponent-1); i0 is
     * chosen by bisection so that w_0 / mean(w) = max_degree / (m/n). */
    double alpha = 1.0 / (exponent - 1.0);
    double target = (double)max_degree / ((double)m / (double)n);
    double lo = 1e-3, hi = (double)n;
    double *w = (double *)malloc(sizeof(double) * n);
    double *cdf = (double *)malloc(sizeof(double) * n);
    uint32_t *perm = (uint32_t *)malloc(sizeof(uint32_t) * n);
    if (!w || !cdf || !perm) {
        free(w);
        free(cdf);
        free(perm);
        return GPMA_ERR_NOMEM;
    }
    for (int it = 0; it < 100; ++it) {
        double mid = 0.5 * (lo + hi), sum = 0;
        for (uint32_t i = 0; i < n; ++i)
            sum += pow((double)i + mid, -alpha);
        double ratio = pow(mid, -alpha) / (sum / n);
        if (ratio > target)
            lo = mid;
        else
            hi = mid;
    }
    double i0 = 0.5 * (lo + hi), total = 0;
    for (uint32_t i = 0; i < n; ++i) {
        w[i] = pow((double)i + i0, -alpha);
        total += w[i];
        cdf[i] = total;
    }
    /* destinations draw from the same weights through a random relabelling,
     * so in-hubs and out-hubs are different nodes; node 0 is the top out-hub */
    {
        xoshiro x;
        xo_seed(&x, seed, 0x9E4Dull);
        for (uint32_t i = 0; i < n; ++i)
            perm[i] = i;
        for (uint32_t i = n; i > 1; --i) {
            uint32_t j = (uint32_t)xo_below(&x, i);
            uint32_t t = perm[i - 1];
            perm[i - 1] = perm[j];
            perm[j] = t;
        }
    }
    uint64_t cap = m + m / 8 + 4096, have = 0, round = 0;
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * cap);
    if (!keys) {
        free(w);
        free(cdf);
        free(perm);
        return GPMA_ERR_NOMEM;
    }
    while (have < m) {
        uint64_t want = (m - have) + (m - have) / 16 + 1024;
        if (have + want > cap) {
            uint64_t ncap = have + want;
            uint64_t *nk = (uint64_t *)realloc(keys, sizeof(uint64_t) * ncap);
            if (!nk) {
                free(keys);
                free(w);
                free(cdf);
                free(perm);
                return GPMA_ERR_NOMEM;
            }
            keys = nk;
            cap = ncap;
        }
        uint64_t chunks = (want + GEN_CHUNK - 1) / GEN_CHUNK;
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t ch = 0; ch < (int64_t)chunks; ++ch) {
            xoshiro x;
            xo_seed(&x, seed, ((round + 1) << 32) + (uint64_t)ch + 1);
            uint64_t l = (uint64_t)ch * GEN_CHUNK, h = l + GEN_CHUNK < want ? l + GEN_CHUNK : want;
            for (uint64_t i = l; i < h; ++i) {
                uint32_t s = pick(cdf, n, xo_unit(&x) * total);
                uint32_t d = perm[pick(cdf, n, xo_unit(&x) * total)];
                keys[have + i] = ((uint64_t)s << 32) | d;
            }
        }
        have = unique_no_loops(keys, have + want);
        ++round;
    }
    shuffle_u64(keys, have, seed);
    split_keys(keys, m, src, dst);
    free(keys);
    free(w);
    free(cdf);
    free(perm);
    return GPMA_OK;
}

gpma_status gpma_edges_to_keys(const uint32_t *src, const uint32_t *dst, uint64_t m, uint64_t *keys) {
    if ((!src || !dst || !keys) && m)
        return GPMA_ERR_INVALID;
    for (uint64_t i = 0; i < m; ++i)
        keys[i] = ((uint64_t)src[i] << 32) + dst[i]; /* gpma_bfs_demo.cu:53 */
    return GPMA_OK;
}

gpma_status gpma_write_edges_text(const char *path, uint32_t n, const uint32_t *src, const uint32_t *dst,
                                  uint64_t m) {
    if (!path || ((!src || !dst) && m))
        return GPMA_ERR_INVALID;
    FILE *f = fopen(path, "w");
    if (!f)
        return GPMA_ERR_IO;
    fprintf(f, "%u %llu\n", n, (unsigned long long)m);
    for (uint64_t i = 0; i < m; ++i)
        fprintf(f, "%u %u\n", src[i], dst[i]);
    return fclose(f) == 0 ? GPMA_OK : GPMA_ERR_IO;
}

gpma_status gpma_read_edges_text(const char *path, uint32_t *n_out, uint64_t *m_out, uint32_t *src, uint32_t *dst,
                                 uint64_t capacity) {
    if (!path || !n_out || !m_out)
        return GPMA_ERR_INVALID;
    FILE *f = fopen(path, "r");
    if (!f)
        return GPMA_ERR_IO;
    unsigned long long n = 0, m = 0;
    if (fscanf(f, "%llu %llu", &n, &m) != 2 || n > 0xFFFFFFFFull) {
        fclose(f);
        return GPMA_ERR_IO;
    }
    *n_out = (uint32_t)n;
    *m_out = m;
    if (!src || !dst) { /* header query */
        fclose(f);
        return GPMA_OK;
    }
    if (capacity < m) {
        fclose(f);
        return GPMA_ERR_INVALID;
    }
    for (uint64_t i = 0; i < m; ++i) {
        unsigned long long x, y;
        if (fscanf(f, "%llu %llu", &x, &y) != 2 || x > 0xFFFFFFFFull || y > 0xFFFFFFFFull) {
            fclose(f);
            return GPMA_ERR_IO;
        }
        src[i] = (uint32_t)x;
        dst[i] = (uint32_t)y;
    }
    fclose(f);
    return GPMA_OK;
}

/* ---- binary edge list ----------------------------------------------------
 * "GPMAEDG1", u32 n, u32 reserved (0), u64 m, m x u32 src, m x u32 dst; all
 * little-endian (written and read byte by byte, so host byte order does not
 * matter). */
static const char EDG_MAGIC[8] = {'G', 'P', 'M', 'A', 'E', 'D', 'G', '1'};

static void put_le(unsigned char *b, uint64_t v, int bytes) {
    for (int i = 0; i < bytes; ++i)
        b[i] = (unsigned char)(v >> (8 * i));
}

static uint64_t get_le(const unsigned char *b, int bytes) {
    uint64_t v = 0;
    for (int i = 0; i < bytes; ++i)
        v |= (uint64_t)b[i] << (8 * i);
    return v;
}

static int write_u32s(FILE *f, const uint32_t *a, uint64_t m) {
    unsigned char buf[4096];
    uint64_t i = 0;
    while (i < m) {
        size_t k = 0;
        for (; k < sizeof(buf) / 4 && i < m; ++k, ++i)
            put_le(buf + 4 * k, a[i], 4);
        if (fwrite(buf, 4, k, f) != k)
            return -1;
    }
    return 0;
}

static int read_u32s(FILE *f, uint32_t *a, uint64_t m) {
    unsigned char buf[4096];
    uint64_t i = 0;
    while (i < m) {
        size_t want = (m - i) < sizeof(buf) / 4 ? (size_t)(m - i) : sizeof(buf) / 4;
        if (fread(buf, 4, want, f) != want)
            return -1;
        for (size_t k = 0; k < want; ++k)
            a[i++] = (uint32_t)get_le(buf + 4 * k, 4);
    }
    return 0;
}

gpma_status gpma_write_edges_bin(const char *path, uint32_t n, const uint32_t *src, const uint32_t *dst, uint64_t m) {
    if (!path || ((!src || !dst) && m))
        return GPMA_ERR_INVALID;
    FILE *f = fopen(path, "wb");
    if (!f)
        return GPMA_ERR_IO;
    unsigned char hdr[24];
    memcpy(hdr, EDG_MAGIC, 8);
    put_le(hdr + 8, n, 4);
    put_le(hdr + 12, 0, 4);
    put_le(hdr + 16, m, 8);
    int bad = fwrite(hdr, 1, sizeof(hdr), f) != sizeof(hdr) || write_u32s(f, src, m) || write_u32s(f, dst, m);
    bad |= fclose(f) != 0;
    return bad ? GPMA_ERR_IO : GPMA_OK;
}

gpma_status gpma_read_edges_bin(const char *path, uint32_t *n_out, uint64_t *m_out, uint32_t *src, uint32_t *dst,
                                uint64_t capacity) {
    if (!path || !n_out || !m_out)
        return GPMA_ERR_INVALID;
    FILE *f = fopen(path, "rb");
    if (!f)
        return GPMA_ERR_IO;
    unsigned char hdr[24];
    if (fread(hdr, 1, sizeof(hdr), f) != sizeof(hdr) || memcmp(hdr, EDG_MAGIC, 8) != 0) {
        fclose(f);
        return GPMA_ERR_IO;
    }
    *n_out = (uint32_t)get_le(hdr + 8, 4);
    *m_out = get_le(hdr + 16, 8);
    if (!src || !dst) { /* header query */
        fclose(f);
        return GPMA_OK;
    }
    if (capacity < *m_out) {
        fclose(f);
        return GPMA_ERR_INVALID;
    }
    int bad = read_u32s(f, src, *m_out) || read_u32s(f, dst, *m_out);
    fclose(f);
    return bad ? GPMA_ERR_IO : GPMA_OK;
}

/* ---- row-range shards ------------------------------------------------------- */

uint32_t gpma_shard_first_row(uint32_t row_num, uint32_t shards, uint32_t s) {
    if (shards == 0)
        return 0;
    if (s > shards)
        s = shards;
    return (uint32_t)(((uint64_t)row_num * s) / shards);
}

/* Shard owning row r: the largest s with first_row(s) <= r, i.e.
 * floor(row_num * s / shards) <= r  <=>  s <= ((r + 1) * shards - 1) / row_num. */
static uint32_t shard_of_row(uint32_t r, uint32_t row_num, uint32_t shards) {
    return (uint32_t)((((uint64_t)r + 1) * shards - 1) / row_num);
}

gpma_status gpma_partition_rows(const uint64_t *keys, const uint8_t *values, uint64_t n, uint32_t row_num,
                                uint32_t shards, int rebase, uint64_t *out_keys, uint8_t *out_values,
                                uint64_t *offsets) {
    if (shards == 0 || row_num == 0 || !offsets || (n && (!keys || !values || !out_keys || !out_values)))
        return GPMA_ERR_INVALID;
    for (uint32_t s = 0; s <= shards; ++s)
        offsets[s] = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const uint32_t r = (uint32_t)(keys[i] >> 32);
        if ((keys[i] >> 32) >= row_num)
            return GPMA_ERR_INVALID;
        offsets[shard_of_row(r, row_num, shards) + 1]++;
    }
    for (uint32_t s = 0; s < shards; ++s)
        offsets[s + 1] += offsets[s];
    uint64_t *cur = (uint64_t *)malloc(sizeof(uint64_t) * shards);
    if (!cur)
        return GPMA_ERR_NOMEM;
    memcpy(cur, offsets, sizeof(uint64_t) * shards);
    for (uint64_t i = 0; i < n; ++i) {
        const uint32_t r = (uint32_t)(keys[i] >> 32);
        const uint32_t s = shard_of_row(r, row_num, shards);
        const uint64_t base = rebase ? gpma_shard_first_row(row_num, shards, s) : 0;
        const uint64_t o = cur[s]++;
        out_keys[o] = ((uint64_t)(r - base) << 32) | (keys[i] & 0xFFFFFFFFull);
        out_values[o] = values[i];
    }
    free(cur);
    return GPMA_OK;
}
