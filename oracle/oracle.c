/*
 * CPU oracle for the lshg engine -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's hot path (peturssonstefan/LSHonGPU,
 * LinearScan/), loop for loop, used by tests/, __graft_entry__.smoke() and the CPU
 * baseline of bench.py as the checker.  The engine never links or calls it.
 *
 * Arithmetic follows the reference's single-precision steps: nvcc contracts
 * `acc += a*b` into fused multiply-adds on the GPU, so those accumulations use fmaf;
 * everything else is rounded step by step (this file is built with
 * -ffp-contract=off).  Selections use the total order (distance, id): ties are broken
 * by the lower index.
 *
 * Pinning: the random generators are checked against the reference's own
 * randomVectorGenerator.cpp compiled here (tests/golden/); the exact-distance oracle
 * against GoldStandard/goldstandard.cpp compiled here (tests/golden/).  The GPU-only
 * steps (sketch bits, cross-polytope keys, rejection samples) are restated from the
 * reference kernels cited at each function; the cuRAND uniforms the sampler consumes
 * are an input (the reference calls curand_init/curand_uniform, CUDA 13.0 headers).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define EMPTY_KEY (~0ull)
#define EMPTY_DIST 2147483648.0f

/* ---------------------------------------------------------------------------
 * keys: (order-preserving float bits << 32) | id
 * ------------------------------------------------------------------------- */
static uint32_t f2o(float f) {
  uint32_t u;
  if (f == 0.0f) f = 0.0f;
  memcpy(&u, &f, 4);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
static float o2f(uint32_t o) {
  uint32_t u = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
  float f;
  memcpy(&f, &u, 4);
  return f;
}
uint64_t or_make_key(float d, int id) { return ((uint64_t)f2o(d) << 32) | (uint32_t)id; }

static int cmp_u64(const void* a, const void* b) {
  uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

/* Keep the `cap` smallest keys of a stream: max-heap of size cap. */
typedef struct {
  uint64_t* h;
  int n, cap;
} heap_t;
static void heap_push(heap_t* H, uint64_t k) {
  if (H->n < H->cap) {
    int i = H->n++;
    H->h[i] = k;
    while (i > 0) {
      int p = (i - 1) / 2;
      if (H->h[p] >= H->h[i]) break;
      uint64_t t = H->h[p]; H->h[p] = H->h[i]; H->h[i] = t;
      i = p;
    }
  } else if (k < H->h[0]) {
    H->h[0] = k;
    int i = 0;
    for (;;) {
      int l = 2 * i + 1, r = l + 1, m = i;
      if (l < H->n && H->h[l] > H->h[m]) m = l;
      if (r < H->n && H->h[r] > H->h[m]) m = r;
      if (m == i) break;
      uint64_t t = H->h[m]; H->h[m] = H->h[i]; H->h[i] = t;
      i = m;
    }
  }
}
/* Sorted ascending into out[cap]; missing entries are EMPTY_KEY. */
static void heap_sorted(heap_t* H, uint64_t* out) {
  qsort(H->h, H->n, 8, cmp_u64);
  for (int i = 0; i < H->cap; ++i) out[i] = i < H->n ? H->h[i] : EMPTY_KEY;
}

static void keys_to_points(const uint64_t* keys, int k, int32_t* ids, float* dists) {
  for (int i = 0; i < k; ++i) {
    if (keys[i] == EMPTY_KEY) { ids[i] = -1; dists[i] = EMPTY_DIST; }
    else { ids[i] = (int32_t)(keys[i] & 0xffffffffu); dists[i] = o2f((uint32_t)(keys[i] >> 32)); }
  }
}

/* ---------------------------------------------------------------------------
 * Host random generators (libstdc++ GCC 13 algorithms used by
 * randomVectorGenerator.cpp:5-87 and weightedMinHash.cuh:231-250)
 * ------------------------------------------------------------------------- */
typedef struct { uint64_t x; } minstd0;
static uint64_t minstd_next(minstd0* g) { g->x = (g->x * 16807ull) % 2147483647ull; return g->x; }
static double canonical53(minstd0* g) {
  const double r = 2147483646.0;
  double sum = 0.0, tmp = 1.0;
  for (int k = 0; k < 2; ++k) {
    double prod = (double)(minstd_next(g) - 1) * tmp;
    sum = sum + prod;
    tmp = tmp * r;
  }
  double ret = sum / tmp;
  if (ret >= 1.0) ret = nextafter(1.0, 0.0);
  return ret;
}
void or_random_normals(int64_t count, double stddev, float* out) {
  minstd0 g = {1};
  int saved_ok = 0;
  double saved = 0;
  for (int64_t i = 0; i < count; ++i) {
    double ret;
    if (saved_ok) { saved_ok = 0; ret = saved; }
    else {
      double x, y, r2;
      do {
        x = 2.0 * canonical53(&g) - 1.0;
        y = 2.0 * canonical53(&g) - 1.0;
        r2 = x * x + y * y;
      } while (r2 > 1.0 || r2 == 0.0);
      double mult = sqrt(-2.0 * log(r2) / r2);
      saved = x * mult;
      saved_ok = 1;
      ret = y * mult;
    }
    out[i] = (float)(ret * stddev + 0.0);
  }
}
static int uniform_int(minstd0* g, int a, int b) {
  const uint64_t urngrange = 2147483645ull, uerange = (uint64_t)(b - a) + 1;
  const uint64_t scaling = urngrange / uerange, past = uerange * scaling;
  uint64_t ret;
  do ret = minstd_next(g) - 1; while (ret >= past);
  return (int)(ret / scaling) + a;
}
void or_random_plus_minus(int64_t count, int32_t* out) {
  minstd0 g = {1};
  for (int64_t i = 0; i < count; ++i) out[i] = uniform_int(&g, 0, 2) == 0 ? -1 : 1;
}
void or_random_bools(int64_t count, uint8_t* out) {
  minstd0 g = {1};
  for (int64_t i = 0; i < count; ++i) out[i] = uniform_int(&g, 0, 1) ? 1 : 0;
}

/* ---------------------------------------------------------------------------
 * Preprocessing
 * ------------------------------------------------------------------------- */
/* transformToUnitVectors (processingUtils.cuh:48-67) */
void or_normalize(float* x, int64_t n, int d) {
  for (int64_t i = 0; i < n; ++i) {
    float m = 0.0f;
    for (int j = 0; j < d; ++j) m = fmaf(x[i * d + j], x[i * d + j], m);
    m = sqrtf(m);
    for (int j = 0; j < d; ++j) x[i * d + j] = x[i * d + j] / m;
  }
}
void or_row_norms(const float* x, int64_t n, int d, float* out) {
  for (int64_t i = 0; i < n; ++i) {
    float m = 0.0f;
    for (int j = 0; j < d; ++j) m = fmaf(x[i * d + j], x[i * d + j], m);
    out[i] = sqrtf(m);
  }
}
/* transformData (processingUtils.cuh:12-46): min of (int)floor over data and
 * queries (starting at 0), then x += |min| on both. */
void or_jaccard_shift(float* x, int64_t n, float* q, int64_t nq, int d) {
  int* mn = (int*)calloc(d, sizeof(int));
  for (int64_t i = 0; i < n; ++i)
    for (int j = 0; j < d; ++j) { int f = (int)floorf(x[i * d + j]); if (f < mn[j]) mn[j] = f; }
  for (int64_t i = 0; i < nq; ++i)
    for (int j = 0; j < d; ++j) { int f = (int)floorf(q[i * d + j]); if (f < mn[j]) mn[j] = f; }
  for (int64_t i = 0; i < n; ++i) for (int j = 0; j < d; ++j) x[i * d + j] = x[i * d + j] + (float)abs(mn[j]);
  for (int64_t i = 0; i < nq; ++i) for (int j = 0; j < d; ++j) q[i * d + j] = q[i * d + j] + (float)abs(mn[j]);
  free(mn);
}

/* ---------------------------------------------------------------------------
 * Distances (distanceFunctions.cuh)
 * ------------------------------------------------------------------------- */
/* angularDistance (:23-40) with magnitudes precomputed by the same chain */
static float angular(const float* q, const float* x, int d, float qn, float xn) {
  float dot = 0.0f;
  for (int j = 0; j < d; ++j) dot = fmaf(q[j], x[j], dot);
  return 1.0f - dot / (qn * xn);
}
/* generalizedJaccardDistance (:10-21) */
static float jaccard(const float* q, const float* x, int d) {
  float mn = 0.0f, mx = 0.0f;
  for (int j = 0; j < d; ++j) {
    mn = mn + fminf(x[j], q[j]);
    mx = mx + fmaxf(x[j], q[j]);
  }
  return 1.0f - mn / mx;
}
/* euclidean (:42-52) -- squared terms accumulated with fmaf (tolerance parity) */
static float sqeuclid(const float* q, const float* x, int d) {
  float acc = 0.0f;
  for (int j = 0; j < d; ++j) { float df = q[j] - x[j]; acc = fmaf(df, df, acc); }
  return acc;
}
static float exact_dist(int dist, const float* q, const float* x, int d, float qn, float xn) {
  if (dist == 1) return angular(q, x, d, qn, xn);
  if (dist == 2) return jaccard(q, x, d);
  if (dist == 3) return sqrtf(sqeuclid(q, x, d));
  return sqeuclid(q, x, d);
}

/* Exact top-k (memOptimizedLinearScan.cu:20-106 semantics, ties by lower index).
 * dist: 1 angular, 2 Jaccard, 3 Euclidean, 4 squared Euclidean. */
void or_exact_topk(const float* x, int64_t n, const float* q, int64_t nq, int d, int dist, int k, int32_t* ids,
                   float* dists) {
  float* xn = (float*)malloc(sizeof(float) * (n > 0 ? n : 1));
  or_row_norms(x, n, d, xn);
  uint64_t* hb = (uint64_t*)malloc(8 * k);
  uint64_t* srt = (uint64_t*)malloc(8 * k);
  for (int64_t qi = 0; qi < nq; ++qi) {
    const float* qr = q + qi * d;
    float qn;
    or_row_norms(qr, 1, d, &qn);
    heap_t H = {hb, 0, k};
    for (int64_t i = 0; i < n; ++i) heap_push(&H, or_make_key(exact_dist(dist, qr, x + i * d, d, qn, xn[i]), (int)i));
    heap_sorted(&H, srt);
    keys_to_points(srt, k, ids + qi * k, dists + qi * k);
  }
  free(xn); free(hb); free(srt);
}

/* FP64 truth: cosine distance 1 - cos in double precision, ties by lower index. */
static void fp64_rows(const float* x, int64_t n, const double* xn, const float* q, int64_t q0, int64_t q1,
                      int64_t qstep, int d, int k, int32_t* ids, double* dists);

static double* fp64_norms(const float* x, int64_t n, int d) {
  double* xn = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
  for (int64_t i = 0; i < n; ++i) {
    double s = 0;
    for (int j = 0; j < d; ++j) s += (double)x[i * d + j] * x[i * d + j];
    xn[i] = sqrt(s);
  }
  return xn;
}

void or_fp64_topk(const float* x, int64_t n, const float* q, int64_t nq, int d, int k, int32_t* ids, double* dists) {
  double* xn = fp64_norms(x, n, d);
  fp64_rows(x, n, xn, q, 0, nq, 1, d, k, ids, dists);
  free(xn);
}

#include <pthread.h>
typedef struct {
  const float *x, *q;
  const double* xn;
  int64_t n, nq, t, nt;
  int d, k;
  int32_t* ids;
  double* dists;
} fp64_job;
static void* fp64_worker(void* a) {
  fp64_job* j = (fp64_job*)a;
  fp64_rows(j->x, j->n, j->xn, j->q, j->t, j->nq, j->nt, j->d, j->k, j->ids, j->dists);
  return NULL;
}
/* Same as or_fp64_topk with queries split over `threads` POSIX threads. */
void or_fp64_topk_mt(const float* x, int64_t n, const float* q, int64_t nq, int d, int k, int threads, int32_t* ids,
                     double* dists) {
  if (threads < 1) threads = 1;
  double* xn = fp64_norms(x, n, d);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * threads);
  fp64_job* jobs = (fp64_job*)malloc(sizeof(fp64_job) * threads);
  for (int t = 0; t < threads; ++t) {
    fp64_job j = {x, q, xn, n, nq, t, threads, d, k, ids, dists};
    jobs[t] = j;
    pthread_create(&th[t], NULL, fp64_worker, &jobs[t]);
  }
  for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
  free(th); free(jobs); free(xn);
}

static void fp64_rows(const float* x, int64_t n, const double* xn, const float* q, int64_t q0, int64_t q1,
                      int64_t qstep, int d, int k, int32_t* ids, double* dists) {
  double* bd = (double*)malloc(sizeof(double) * k);
  int32_t* bi = (int32_t*)malloc(sizeof(int32_t) * k);
  for (int64_t qi = q0; qi < q1; qi += qstep) {
    const float* qr = q + qi * d;
    double qs = 0;
    for (int j = 0; j < d; ++j) qs += (double)qr[j] * qr[j];
    double qn = sqrt(qs);
    int cnt = 0;
    for (int64_t i = 0; i < n; ++i) {
      double dot = 0;
      for (int j = 0; j < d; ++j) dot += (double)qr[j] * x[i * d + j];
      double dd = 1.0 - dot / (qn * xn[i]);
      /* insertion into sorted (dd, id) list of length <= k */
      if (cnt == k && !(dd < bd[k - 1])) continue;
      int pos = cnt < k ? cnt : k - 1;
      while (pos > 0 && (bd[pos - 1] > dd)) { if (pos < k) { bd[pos] = bd[pos - 1]; bi[pos] = bi[pos - 1]; } --pos; }
      bd[pos] = dd; bi[pos] = (int32_t)i;
      if (cnt < k) ++cnt;
    }
    for (int i = 0; i < k; ++i) {
      ids[qi * k + i] = i < cnt ? bi[i] : -1;
      dists[qi * k + i] = i < cnt ? bd[i] : INFINITY;
    }
  }
  free(bd); free(bi);
}

/* ---------------------------------------------------------------------------
 * Sketch builders
 * ------------------------------------------------------------------------- */
/* SimHash (simHash.cuh:20-46): plane p = w*bits + b, bit b of word w = (dot >= 0) */
void or_simhash(const float* x, int64_t n, int d, const float* planes, int words, int bits, uint32_t* out) {
  for (int64_t i = 0; i < n; ++i)
    for (int w = 0; w < words; ++w) {
      uint32_t s = 0;
      for (int b = 0; b < bits; ++b) {
        const float* r = planes + ((int64_t)w * bits + b) * d;
        float dot = 0.0f;
        for (int j = 0; j < d; ++j) dot = fmaf(x[i * d + j], r[j], dot);
        s |= (uint32_t)(dot >= 0 ? 1 : 0) << b;
      }
      out[i * words + w] = s;
    }
}
/* JL (simHashJL.cuh:34-51) */
void or_jl(const float* x, int64_t n, int d, const float* R, int sdim, float* out) {
  for (int64_t i = 0; i < n; ++i)
    for (int s = 0; s < sdim; ++s) {
      float dot = 0.0f;
      for (int j = 0; j < d; ++j) dot = fmaf(x[i * d + j], R[(int64_t)s * d + j], dot);
      out[i * sdim + s] = dot;
    }
}
/* Cross-polytope (crossPolyTope.cuh:25-85); hashes > 1 concatenates (key*2P + h). */
void or_crosspoly(const float* x, int64_t n, int d, int P, int tables, int hashes, int rounds, const int32_t* diag,
                  uint16_t* keys) {
  float* v = (float*)malloc(sizeof(float) * P);
  float* t = (float*)malloc(sizeof(float) * P);
  for (int64_t i = 0; i < n; ++i)
    for (int tb = 0; tb < tables; ++tb) {
      uint32_t key = 0;
      for (int h = 0; h < hashes; ++h) {
        for (int p = 0; p < P; ++p) v[p] = p < d ? x[i * d + p] : 0.0f;
        for (int r = 0; r < rounds; ++r) {
          const int32_t* D = diag + (((int64_t)tb * hashes + h) * rounds + r) * P;
          for (int p = 0; p < P; ++p) v[p] = v[p] * (float)D[p];
          for (int o = P / 2; o > 0; o /= 2) {
            for (int p = 0; p < P; ++p) {
              int q = p ^ o;
              t[p] = p < q ? v[p] + v[q] : -v[p] + v[q];
            }
            memcpy(v, t, sizeof(float) * P);
          }
        }
        int index = 0;
        float total = (float)INT32_MIN;
        for (int p = 0; p < P; ++p) {
          int neg = v[p] < 0;
          float mv = neg ? fmaxf(total, -v[p]) : fmaxf(total, v[p]);
          if (mv > total) { index = neg ? p : p + P; total = mv; }
        }
        key = key * (uint32_t)(2 * P) + (uint32_t)index;
      }
      keys[i * tables + tb] = (uint16_t)key;
    }
  free(v); free(t);
}

/* Weighted MinHash bounds and map (weightedMinHash.cuh:41-90): m[d] = max ceil over data
 * and queries (from 0), start = prefix, map[slot] = dim.  Returns M. */
int or_wmh_bounds(const float* x, int64_t n, const float* q, int64_t nq, int d, int32_t* start, int32_t* map,
                  int map_cap) {
  int* m = (int*)calloc(d, sizeof(int));
  for (int64_t i = 0; i < n; ++i)
    for (int j = 0; j < d; ++j) { int c = (int)ceilf(x[i * d + j]); if (c > m[j]) m[j] = c; }
  for (int64_t i = 0; i < nq; ++i)
    for (int j = 0; j < d; ++j) { int c = (int)ceilf(q[i * d + j]); if (c > m[j]) m[j] = c; }
  int M = 0;
  for (int j = 0; j < d; ++j) {
    start[j] = M;
    for (int s = 0; s < m[j]; ++s) { if (M < map_cap) map[M] = j; ++M; }
  }
  free(m);
  return M;
}

/* Rejection samples (weightedMinHash.cuh:98-166) from given uniforms u[h*T + j]
 * (the values curand_uniform returns after curand_init(seed_h, 0, 10000)).
 * Returns the number of samples that needed more than T draws (then output 0). */
int64_t or_wmh_sketch(const float* x, int64_t n, int d, const int32_t* start, const int32_t* map, int M,
                      const float* u, int H, int T, int onebit, int words, int hashBits, const uint8_t* bitmap,
                      int bitmapLen, uint8_t* out8, uint32_t* out32) {
  int64_t over = 0;
  const float Mf = (float)M;
  for (int64_t i = 0; i < n; ++i) {
    const float* xi = x + i * d;
    for (int g = 0; g < (onebit ? words : H); ++g) {
      uint32_t word = 0;
      for (int b = 0; b < (onebit ? hashBits : 1); ++b) {
        int h = onebit ? g * hashBits + b : g;
        int cnt = 0, found = 0;
        for (int j = 0; j < T; ++j) {
          float r = Mf * u[(int64_t)h * T + j];
          int ri = (int)r;
          if (ri < M) {
            int c = map[ri];
            if (r <= (float)start[c] + xi[c]) { found = 1; break; }
          }
          ++cnt;
        }
        if (!found) { ++over; cnt = 0; }
        if (onebit) word |= (uint32_t)((cnt < bitmapLen && bitmap[cnt]) ? 1 : 0) << b;
        else out8[i * H + h] = (uint8_t)(cnt & 255);
      }
      if (onebit) out32[i * words + g] = word;
    }
  }
  return over;
}

/* ---------------------------------------------------------------------------
 * Consistent weighted sampling (implementation 10; no reference counterpart).
 * Restates the engine's sketch (lshongpu_gb300/csrc/cws.cu) from the published
 * algorithm -- Ioffe, "Improved Consistent Sampling, Weighted Minhash and L1
 * Sketching", ICDM 2010 -- with the engine's draw table and single-precision steps:
 *   t_i = floor(ln S_i * (1/r) + beta),  ln a_i = ln c - r ((t_i - beta) + 1),
 *   sample = (argmin_i ln a_i (lowest i on ties), t_i*), (d, 0) for no positive entry.
 * Draws: splitmix64 (Steele, Lea, Flood, OOPSLA 2014) as a counter hash.  This file is
 * built with -ffp-contract=off, so each float operation below is rounded on its own, as
 * the device code's __f*_rn intrinsics are.
 * ------------------------------------------------------------------------- */
#define CWS_SEED 0x6C7368672D637773ull

static uint64_t cws_mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

#define CWS_KEY_SEED 0x6C7368672D6B6579ull

static double cws_uniform(uint64_t seed, int j, int i, int m) {
  uint64_t c = ((uint64_t)j * 65536u + (uint64_t)i) * 8u + (uint64_t)m;
  uint64_t z = cws_mix(seed + (c + 1) * 0x9E3779B97F4A7C15ull);
  return ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

/* table [d][S][4]: r, 1/r, ln c, beta (r, c ~ Gamma(2, 1) as sums of two Exp(1));
 * key = 1: the draws of LSH keys (keysImplementation 10), independent of the sketch's */
void or_cws_tables_seeded(int d, int S, int key, float* tab) {
  const uint64_t seed = key ? CWS_KEY_SEED : CWS_SEED;
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < S; ++j) {
      double r = -(log(cws_uniform(seed, j, i, 0)) + log(cws_uniform(seed, j, i, 1)));
      double c = -(log(cws_uniform(seed, j, i, 2)) + log(cws_uniform(seed, j, i, 3)));
      float rf = (float)r;
      float* t = tab + ((size_t)i * S + j) * 4;
      t[0] = rf;
      t[1] = 1.0f / rf;
      t[2] = (float)log(c);
      t[3] = (float)cws_uniform(seed, j, i, 4);
    }
}
void or_cws_tables(int d, int S, float* tab) { or_cws_tables_seeded(d, S, 0, tab); }

/* LSH keys [n][L] from samples [n][L*K][2]: table t folds its K samples into a 64-bit
 * hash (h = mix(h ^ (index << 32 | t)), starting from golden * (t + 1)) and keeps the top
 * `bits` bits. */
void or_cws_keys(const int32_t* smp, int64_t n, int L, int K, int bits, uint16_t* keys) {
  for (int64_t r = 0; r < n; ++r)
    for (int t = 0; t < L; ++t) {
      uint64_t h = 0x9E3779B97F4A7C15ull * (uint64_t)(t + 1);
      for (int j = 0; j < K; ++j) {
        const int32_t* v = smp + ((r * L + t) * (int64_t)K + j) * 2;
        h = cws_mix(h ^ (((uint64_t)(uint32_t)v[0] << 32) | (uint32_t)v[1]));
      }
      keys[r * L + t] = (uint16_t)(h >> (64 - bits));
    }
}

/* ln x for positive finite x: x = m 2^e, m in [sqrt(1/2), sqrt(2)], ln m = 2 atanh(s),
 * s = (m - 1)/(m + 1), the atanh series to s^9, ln2 split in a high and a low part. */
float or_cws_logf(float x) {
  int e = 0;
  uint32_t u;
  memcpy(&u, &x, 4);
  if (u < 0x00800000u) {
    float y = x * 16777216.0f;
    memcpy(&u, &y, 4);
    e = -24;
  }
  e += (int)(u >> 23) - 127;
  uint32_t mu = (u & 0x007FFFFFu) | 0x3F800000u;
  float m;
  memcpy(&m, &mu, 4);
  if (m > 1.41421354f) {
    m = m * 0.5f;
    e += 1;
  }
  float s = (m - 1.0f) / (m + 1.0f);
  float z = s * s;
  float p = 0.222222224f;
  p = p * z + 0.285714298f;
  p = p * z + 0.400000006f;
  p = p * z + 0.666666687f;
  p = p * z + 2.0f;
  float lnm = p * s;
  float ef = (float)e;
  return ef * 0.693145752f + (ef * 1.42860677e-06f + lnm);
}

/* samples [n][S] of (index, t) int32 pairs */
void or_cws_sketch(const float* x, int64_t n, int d, int S, const float* tab, int32_t* out) {
  float* L = (float*)malloc(sizeof(float) * (size_t)d);
  for (int64_t r = 0; r < n; ++r) {
    for (int i = 0; i < d; ++i) {
      float v = x[r * d + i];
      L[i] = (v > 0.0f && v < INFINITY) ? or_cws_logf(v) : INFINITY;
    }
    for (int j = 0; j < S; ++j) {
      float best = INFINITY;
      int bk = d, bt = 0;
      for (int i = 0; i < d; ++i) {
        if (L[i] == INFINITY) continue;
        const float* T = tab + ((size_t)i * S + j) * 4;
        float v = L[i] * T[1] + T[3];
        v = fminf(fmaxf(v, -1.0e9f), 1.0e9f);
        float tf = floorf(v);
        float la = T[2] - T[0] * ((tf - T[3]) + 1.0f);
        if (la < best) {
          best = la;
          bk = i;
          bt = (int)tf;
        }
      }
      out[(r * S + j) * 2] = bk;
      out[(r * S + j) * 2 + 1] = bt;
    }
  }
  free(L);
}

/* ---------------------------------------------------------------------------
 * Sketched scans: top-C by (sketch distance, id), exact re-rank, top-k
 * (sketchedDistanceScanners.cuh, candidateSetScanner.cuh)
 * kind: 3 Hamming words, 4 byte sketches, 5 one-bit words, 6 JL floats,
 * 10 CWS (index, t) pairs (width = samples)
 * ------------------------------------------------------------------------- */
static float sketch_dist(int kind, const void* xs, const void* qs, int64_t i, int64_t qi, int width) {
  if (kind == 10) {
    const int32_t* a = (const int32_t*)xs + i * width * 2;
    const int32_t* b = (const int32_t*)qs + qi * width * 2;
    int m = 0;
    for (int w = 0; w < width; ++w) m += (a[2 * w] == b[2 * w] && a[2 * w + 1] == b[2 * w + 1]) ? 1 : 0;
    return 1.0f - (float)m / (float)width;
  }
  if (kind == 6) {
    const float* a = (const float*)xs + i * width;
    const float* b = (const float*)qs + qi * width;
    return sqeuclid(b, a, width);
  }
  if (kind == 4) {
    const uint8_t* a = (const uint8_t*)xs + i * width;
    const uint8_t* b = (const uint8_t*)qs + qi * width;
    float sim = 0;
    for (int w = 0; w < width; ++w) sim += a[w] == b[w] ? 1 : 0;
    sim /= (float)width;
    return 1.0f - sim;
  }
  const uint32_t* a = (const uint32_t*)xs + i * width;
  const uint32_t* b = (const uint32_t*)qs + qi * width;
  int hd = 0;
  for (int w = 0; w < width; ++w) hd += __builtin_popcount(a[w] ^ b[w]);
  if (kind == 3) return (float)hd;
  float sim = 0;
  for (int w = 0; w < width; ++w) sim += (float)(32 - __builtin_popcount(a[w] ^ b[w]));
  sim /= (float)(32 * width);
  return 1.0f - sim;
}

/* candidates out (optional): [nq][C] sorted keys.  Final: ids/dists [nq][k]. */
void or_sketch_scan(const float* x, int64_t n, const float* q, int64_t nq, int d, int kind, const void* xs,
                    const void* qs, int width, int C, int dist, int k, uint64_t* cand_out, int32_t* ids, float* dists) {
  float* xn = (float*)malloc(sizeof(float) * n);
  or_row_norms(x, n, d, xn);
  uint64_t* hb = (uint64_t*)malloc(8 * C);
  uint64_t* cand = (uint64_t*)malloc(8 * C);
  uint64_t* fin = (uint64_t*)malloc(8 * (C > k ? C : k));
  for (int64_t qi = 0; qi < nq; ++qi) {
    heap_t H = {hb, 0, C};
    for (int64_t i = 0; i < n; ++i) heap_push(&H, or_make_key(sketch_dist(kind, xs, qs, i, qi, width), (int)i));
    heap_sorted(&H, cand);
    if (cand_out) memcpy(cand_out + qi * C, cand, 8 * C);
    const float* qr = q + qi * d;
    float qn;
    or_row_norms(qr, 1, d, &qn);
    int m = 0;
    for (int c = 0; c < C; ++c) {
      if (cand[c] == EMPTY_KEY) continue;
      int id = (int)(cand[c] & 0xffffffffu);
      fin[m++] = or_make_key(exact_dist(dist, qr, x + (int64_t)id * d, d, qn, xn[id]), id);
    }
    qsort(fin, m, 8, cmp_u64);
    for (int i = m; i < k; ++i) fin[i] = EMPTY_KEY;
    keys_to_points(fin, k, ids + qi * k, dists + qi * k);
  }
  free(xn); free(hb); free(cand); free(fin);
}

/* ---------------------------------------------------------------------------
 * (K,L) LSH (lshFramework.cuh:102-280)
 * ------------------------------------------------------------------------- */
/* CSR buckets: offsets[t*S + key] absolute (table t starts at t*n); ids ascending. */
void or_lsh_build(const uint16_t* keys, int64_t n, int tables, int S, int32_t* offsets, int32_t* buckets) {
  memset(offsets, 0, sizeof(int32_t) * (size_t)tables * S);
  for (int64_t i = 0; i < n; ++i)
    for (int t = 0; t < tables; ++t) offsets[(int64_t)t * S + keys[i * tables + t]]++;
  for (int t = 0; t < tables; ++t) {
    int run = (int)(t * n);
    for (int s = 0; s < S; ++s) { int c = offsets[(int64_t)t * S + s]; offsets[(int64_t)t * S + s] = run; run += c; }
  }
  int32_t* cur = (int32_t*)malloc(sizeof(int32_t) * (size_t)tables * S);
  memcpy(cur, offsets, sizeof(int32_t) * (size_t)tables * S);
  for (int64_t i = 0; i < n; ++i)
    for (int t = 0; t < tables; ++t) buckets[cur[(int64_t)t * S + keys[i * tables + t]]++] = (int32_t)i;
  free(cur);
}

/* Query: distinct candidates from the L buckets; exact distances (sketched = 0) or
 * top-C by sketch distance then exact re-rank; top-k by (distance, id). */
void or_lsh_query(const float* x, int64_t n, const float* q, int64_t nq, int d, const uint16_t* qkeys, int tables,
                  int S, const int32_t* offsets, const int32_t* buckets, int sketched, int kind, const void* xs,
                  const void* qs, int width, int C, int dist, int k, int32_t* ids, float* dists) {
  float* xn = (float*)malloc(sizeof(float) * n);
  or_row_norms(x, n, d, xn);
  uint8_t* seen = (uint8_t*)calloc(n, 1);
  int64_t* list = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
  int cap = sketched ? C : k;
  uint64_t* hb = (uint64_t*)malloc(8 * (cap > k ? cap : k));
  uint64_t* srt = (uint64_t*)malloc(8 * (cap > k ? cap : k));
  for (int64_t qi = 0; qi < nq; ++qi) {
    const float* qr = q + qi * d;
    float qn;
    or_row_norms(qr, 1, d, &qn);
    int64_t m = 0;
    for (int t = 0; t < tables; ++t) {
      int key = qkeys[qi * tables + t];
      if (key >= S) continue;
      int st = offsets[(int64_t)t * S + key];
      int en = key >= S - 1 ? (int)(t * n + n) : offsets[(int64_t)t * S + key + 1];
      for (int b = st; b < en; ++b) {
        int id = buckets[b];
        if (!seen[id]) { seen[id] = 1; list[m++] = id; }
      }
    }
    heap_t H = {hb, 0, cap};
    for (int64_t c = 0; c < m; ++c) {
      int id = (int)list[c];
      float dd = sketched ? sketch_dist(kind, xs, qs, id, qi, width) : exact_dist(dist, qr, x + (int64_t)id * d, d, qn, xn[id]);
      heap_push(&H, or_make_key(dd, id));
    }
    heap_sorted(&H, srt);
    if (sketched) {
      heap_t H2 = {hb, 0, k};
      for (int c = 0; c < cap; ++c) {
        if (srt[c] == EMPTY_KEY) continue;
        int id = (int)(srt[c] & 0xffffffffu);
        heap_push(&H2, or_make_key(exact_dist(dist, qr, x + (int64_t)id * d, d, qn, xn[id]), id));
      }
      uint64_t* fin = (uint64_t*)malloc(8 * k);
      heap_sorted(&H2, fin);
      keys_to_points(fin, k, ids + qi * k, dists + qi * k);
      free(fin);
    } else {
      keys_to_points(srt, k, ids + qi * k, dists + qi * k);
    }
    for (int64_t c = 0; c < m; ++c) seen[list[c]] = 0;
  }
  free(xn); free(seen); free(list); free(hb); free(srt);
}
