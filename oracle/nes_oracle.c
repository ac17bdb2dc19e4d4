/*
 * nes_oracle.c -- CPU oracle for the render-and-encode hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the test suite, the
 * smoke entry and the CPU-baseline leg of the benchmark call it to produce the
 * answers the CUDA library must reproduce.  Nothing in the product links it.
 *
 * What it restates (each function names the reference call site it follows):
 *
 *  - The renderer that neserver asks for a frame over TCP
 *    (src/server.cpp:161-194; the renderer itself is the un-vendored,
 *    unpinned moonsikpark/instant-ngp-renderer, README.md:5).  Its math is the
 *    published Instant-NGP method (Mueller, Evans, Schied, Keller, "Instant
 *    Neural Graphics Primitives with a Multiresolution Hash Encoding",
 *    SIGGRAPH 2022): multiresolution hash grid, tiny MLPs, occupancy-grid ray
 *    march, emission-absorption compositing.  Every free choice of that method
 *    is fixed by the scene specification written out below and computed here
 *    in FP64 (ray set-up excepted, see oracle_ray_setup).
 *    PARITY UNPINNED: the reference ships no renderer, no golden image and no
 *    test for this path, so nothing here is checked against reference output.
 *    It is pinned instead by known-answer tests of its parts (hash indices
 *    worked by hand from the primes, the resolution table, trilinear weights,
 *    spherical-harmonic orthonormality).
 *
 *  - RenderedFrame::convert_frame (include/base/video/rendered_frame.h:24-33),
 *    i.e. libswscale RGB24->YUV420P and GRAY8->YUV420P at the frame's own
 *    size (src/base/video/type_managers.cc:143-153).  libswscale is not
 *    installed in this container nor on the GPU host, so this is the repo's
 *    own integer restatement of ITU-R BT.601 studio-range conversion with
 *    2x2 chroma averaging.  SWSCALE PARITY UNPINNED; the restatement is pinned
 *    by the published 100% colour-bar YCbCr values of BT.601.
 *
 *  - Depth packing FP32 scene units -> uint16 millimetres (new in the
 *    GB300 build; the reference ships GRAY8 depth, src/server.cpp:193-194).
 *
 * Build: oracle/build_oracle.py (gcc -O2 -ffp-contract=off, no fast-math:
 * the FP32 ray set-up must round exactly like the CUDA kernels' *_rn ops).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* Scene specification                                                  */
/* ------------------------------------------------------------------ */
#define OR_LEVELS 16
#define OR_FEATS 2
#define OR_ENC (OR_LEVELS * OR_FEATS) /* 32 */
#define OR_HID 64
#define OR_DOUT 16
#define OR_CIN 32 /* 16 SH + 15 geometry features + 1 zero pad */
#define OR_OCC_RES 128
#define OR_MAX_STEPS 1024
#define OR_OCC_THRESHOLD 0.01
#define OR_T_STOP 1e-4

/* Per-level grid resolution N_l = floor(16 * b^l), b = (2048/16)^(1/15),
 * fixed once as integers so every implementation shares it. */
static const int OR_RES[OR_LEVELS] = {16,  22,  30,  42,  58,   80,   111,  153,
                                      212, 294, 406, 561, 776, 1072, 1482, 2048};
/* Spatial-hash primes of the Instant-NGP paper (one per axis). */
static const uint32_t OR_PRIME[3] = {1u, 2654435761u, 805459861u};
/* March step sqrt(3)/1024 rounded once to FP32 (= 0x1.bb67aep-10). */
static const float OR_DT = 0x1.bb67aep-10f;

/* ------------------------------------------------------------------ */
/* SplitMix64 (Steele, Lea, Flood, OOPSLA 2014), counter form.          */
/* Draw i of stream s under seed: mix(key + (i+1)*GAMMA),               */
/* key = mix(seed * 256 + s).                                           */
/* ------------------------------------------------------------------ */
#define OR_GAMMA 0x9E3779B97F4A7C15ull
static inline uint64_t or_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
uint64_t oracle_stream_key(uint64_t seed, uint32_t stream) {
  return or_mix64(seed * 256ull + stream);
}
static inline uint64_t or_draw(uint64_t key, uint64_t i) {
  return or_mix64(key + (i + 1ull) * OR_GAMMA);
}
/* 24-bit uniform integer in [0, 2^24). */
static inline uint32_t or_u24(uint64_t key, uint64_t i) {
  return (uint32_t)(or_draw(key, i) >> 40);
}

enum { OR_S_TABLE = 0, OR_S_DW1 = 1, OR_S_DW2 = 2, OR_S_CW1 = 3, OR_S_CW2 = 4, OR_S_CW3 = 5 };

typedef struct {
  uint32_t log2T, T;
  float *table;    /* [16][T][2] */
  float dw1[OR_HID * OR_ENC];   /* density 32->64, row-major [out][in] */
  float dw2[OR_DOUT * OR_HID];  /* density 64->16 */
  float cw1[OR_HID * OR_CIN];   /* colour 31(+pad)->64, column 31 is zero */
  float cw2[OR_HID * OR_HID];   /* colour 64->64 */
  float cw3[3 * OR_HID];        /* colour 64->3 */
} or_scene;

/* Xavier-uniform weight: U(-a, a), a = sqrt(6 / (fan_in + fan_out)). */
static float or_xavier(uint64_t key, uint64_t i, int fan_in, int fan_out) {
  double a = sqrt(6.0 / (double)(fan_in + fan_out));
  double u = (double)or_u24(key, i) * 0x1p-23 - 1.0; /* exact, in [-1, 1) */
  return (float)(u * a);
}

static void or_fill_dense(float *w, int rows, int cols, int fan_in, int fan_out,
                          uint64_t key) {
  for (int r = 0; r < rows; r++)
    for (int c = 0; c < cols; c++)
      w[r * cols + c] = or_xavier(key, (uint64_t)r * cols + c, fan_in, fan_out);
}

void *oracle_scene_new(uint64_t seed, uint32_t log2T) {
  if (log2T < 10 || log2T > 24) return NULL;
  or_scene *s = (or_scene *)calloc(1, sizeof(or_scene));
  if (!s) return NULL;
  s->log2T = log2T;
  s->T = 1u << log2T;
  size_t n = (size_t)OR_LEVELS * s->T * OR_FEATS;
  s->table = (float *)malloc(n * sizeof(float));
  if (!s->table) {
    free(s);
    return NULL;
  }
  uint64_t kt = oracle_stream_key(seed, OR_S_TABLE);
  for (size_t i = 0; i < n; i++) /* U(-0.5, 0.5), exact in FP32 */
    s->table[i] = (float)((int32_t)or_u24(kt, i) - (1 << 23)) * 0x1p-24f;
  or_fill_dense(s->dw1, OR_HID, OR_ENC, OR_ENC, OR_HID, oracle_stream_key(seed, OR_S_DW1));
  or_fill_dense(s->dw2, OR_DOUT, OR_HID, OR_HID, OR_DOUT, oracle_stream_key(seed, OR_S_DW2));
  {
    uint64_t k = oracle_stream_key(seed, OR_S_CW1);
    for (int r = 0; r < OR_HID; r++) {
      for (int c = 0; c < 31; c++)
        s->cw1[r * OR_CIN + c] = or_xavier(k, (uint64_t)r * 31 + c, 31, OR_HID);
      s->cw1[r * OR_CIN + 31] = 0.0f;
    }
  }
  or_fill_dense(s->cw2, OR_HID, OR_HID, OR_HID, OR_HID, oracle_stream_key(seed, OR_S_CW2));
  or_fill_dense(s->cw3, 3, OR_HID, OR_HID, 3, oracle_stream_key(seed, OR_S_CW3));
  return s;
}

void oracle_scene_free(void *h) {
  or_scene *s = (or_scene *)h;
  if (!s) return;
  free(s->table);
  free(s);
}

/* Export the scene parameters (for byte-equality tests against the product's
 * generator).  which: 0 table, 1 dw1, 2 dw2, 3 cw1, 4 cw2, 5 cw3. */
const float *oracle_scene_param(void *h, int which, size_t *count) {
  or_scene *s = (or_scene *)h;
  switch (which) {
    case 0: *count = (size_t)OR_LEVELS * s->T * OR_FEATS; return s->table;
    case 1: *count = OR_HID * OR_ENC; return s->dw1;
    case 2: *count = OR_DOUT * OR_HID; return s->dw2;
    case 3: *count = OR_HID * OR_CIN; return s->cw1;
    case 4: *count = OR_HID * OR_HID; return s->cw2;
    case 5: *count = 3 * OR_HID; return s->cw3;
  }
  *count = 0;
  return NULL;
}

/* Overwrite a parameter array (used by the gradient tests to perturb one
 * parameter for finite differences). */
int oracle_scene_set_param(void *h, int which, const float *src, size_t count) {
  size_t n;
  float *dst = (float *)oracle_scene_param(h, which, &n);
  if (!dst || n != count) return -1;
  memcpy(dst, src, n * sizeof(float));
  return 0;
}

void oracle_resolutions(int *out16) { memcpy(out16, OR_RES, sizeof(OR_RES)); }
float oracle_dt(void) { return OR_DT; }

/* ------------------------------------------------------------------ */
/* Hash-grid index (Instant-NGP paper, Sec. 3): a level whose (N+1)^3   */
/* vertices fit in T entries is indexed densely (x-fastest), otherwise  */
/* by the XOR of coordinate*prime, modulo T.                            */
/* ------------------------------------------------------------------ */
uint32_t oracle_grid_index(uint32_t level, uint32_t T, uint32_t x, uint32_t y, uint32_t z) {
  uint64_t side = (uint64_t)OR_RES[level] + 1;
  if (side * side * side <= (uint64_t)T)
    return (uint32_t)(x + side * (y + side * z));
  uint32_t h = (x * OR_PRIME[0]) ^ (y * OR_PRIME[1]) ^ (z * OR_PRIME[2]);
  return h & (T - 1u);
}

/* Encode one position x in [0,1]^3 into 32 features (level-major). */
void oracle_encode(const void *h, const double *x, double *feat) {
  const or_scene *s = (const or_scene *)h;
  for (int l = 0; l < OR_LEVELS; l++) {
    int N = OR_RES[l];
    double f[3];
    uint32_t i0[3];
    for (int a = 0; a < 3; a++) {
      double p = x[a] * (double)N;
      double fl = floor(p);
      if (fl < 0.0) fl = 0.0;
      if (fl > (double)(N - 1)) fl = (double)(N - 1);
      i0[a] = (uint32_t)fl;
      f[a] = p - fl;
    }
    double acc0 = 0.0, acc1 = 0.0;
    const float *tab = s->table + (size_t)l * s->T * OR_FEATS;
    for (int c = 0; c < 8; c++) {
      int dx = c & 1, dy = (c >> 1) & 1, dz = (c >> 2) & 1;
      double w = (dx ? f[0] : 1.0 - f[0]) * (dy ? f[1] : 1.0 - f[1]) *
                 (dz ? f[2] : 1.0 - f[2]);
      uint32_t idx = oracle_grid_index((uint32_t)l, s->T, i0[0] + dx, i0[1] + dy, i0[2] + dz);
      acc0 += w * (double)tab[(size_t)idx * 2 + 0];
      acc1 += w * (double)tab[(size_t)idx * 2 + 1];
    }
    feat[2 * l + 0] = acc0;
    feat[2 * l + 1] = acc1;
  }
}

/* Real spherical harmonics, bands 0..3 (16 functions), orthonormal on the
 * unit sphere; standard closed forms in Cartesian coordinates. */
void oracle_sh16(const double *d, double *sh) {
  const double PI = 3.14159265358979323846;
  double x = d[0], y = d[1], z = d[2];
  double c0 = 0.5 * sqrt(1.0 / PI), c1 = sqrt(3.0 / (4.0 * PI));
  double c2a = 0.5 * sqrt(15.0 / PI), c2b = 0.25 * sqrt(5.0 / PI), c2c = 0.25 * sqrt(15.0 / PI);
  double c3a = 0.25 * sqrt(35.0 / (2.0 * PI)), c3b = 0.5 * sqrt(105.0 / PI);
  double c3c = 0.25 * sqrt(21.0 / (2.0 * PI)), c3d = 0.25 * sqrt(7.0 / PI);
  double c3e = 0.25 * sqrt(105.0 / PI);
  sh[0] = c0;
  sh[1] = c1 * y;
  sh[2] = c1 * z;
  sh[3] = c1 * x;
  sh[4] = c2a * x * y;
  sh[5] = c2a * y * z;
  sh[6] = c2b * (3.0 * z * z - 1.0);
  sh[7] = c2a * x * z;
  sh[8] = c2c * (x * x - y * y);
  sh[9] = c3a * y * (3.0 * x * x - y * y);
  sh[10] = c3b * x * y * z;
  sh[11] = c3c * y * (5.0 * z * z - 1.0);
  sh[12] = c3d * z * (5.0 * z * z - 3.0);
  sh[13] = c3c * x * (5.0 * z * z - 1.0);
  sh[14] = c3e * z * (x * x - y * y);
  sh[15] = c3a * x * (x * x - 3.0 * y * y);
}

static inline double or_relu(double v) { return v > 0.0 ? v : 0.0; }

/* Density MLP 32->64(ReLU)->16, no biases.  out[0] is the density logit. */
static void or_density(const or_scene *s, const double *enc, double *h1, double *out) {
  for (int j = 0; j < OR_HID; j++) {
    double a = 0.0;
    for (int k = 0; k < OR_ENC; k++) a += (double)s->dw1[j * OR_ENC + k] * enc[k];
    h1[j] = or_relu(a);
  }
  for (int m = 0; m < OR_DOUT; m++) {
    double a = 0.0;
    for (int j = 0; j < OR_HID; j++) a += (double)s->dw2[m * OR_HID + j] * h1[j];
    out[m] = a;
  }
}

/* Colour MLP [SH16 | dens_out[1..15] | 0] 32->64->64->3, ReLU, sigmoid. */
static void or_colour(const or_scene *s, const double *cin, double *g1, double *g2,
                      double *rgb) {
  for (int j = 0; j < OR_HID; j++) {
    double a = 0.0;
    for (int k = 0; k < OR_CIN; k++) a += (double)s->cw1[j * OR_CIN + k] * cin[k];
    g1[j] = or_relu(a);
  }
  for (int j = 0; j < OR_HID; j++) {
    double a = 0.0;
    for (int k = 0; k < OR_HID; k++) a += (double)s->cw2[j * OR_HID + k] * g1[k];
    g2[j] = or_relu(a);
  }
  for (int c = 0; c < 3; c++) {
    double a = 0.0;
    for (int k = 0; k < OR_HID; k++) a += (double)s->cw3[c * OR_HID + k] * g2[k];
    rgb[c] = 1.0 / (1.0 + exp(-a));
  }
}

/* Full field query: density sigma and colour at x seen along d. */
void oracle_query(const void *h, const double *x, const double *d, double *sigma, double *rgb) {
  const or_scene *s = (const or_scene *)h;
  double enc[OR_ENC], h1[OR_HID], out[OR_DOUT], cin[OR_CIN], g1[OR_HID], g2[OR_HID];
  oracle_encode(h, x, enc);
  or_density(s, enc, h1, out);
  *sigma = exp(out[0] - 1.0);
  oracle_sh16(d, cin);
  for (int i = 0; i < 15; i++) cin[16 + i] = out[1 + i];
  cin[31] = 0.0;
  or_colour(s, cin, g1, g2, rgb);
}

double oracle_density(const void *h, const double *x) {
  const or_scene *s = (const or_scene *)h;
  double enc[OR_ENC], h1[OR_HID], out[OR_DOUT];
  oracle_encode(h, x, enc);
  or_density(s, enc, h1, out);
  return exp(out[0] - 1.0);
}

/* ------------------------------------------------------------------ */
/* Ray set-up, in FP32 with a fixed operation order (no fused multiply- */
/* add), identical in the CUDA kernels: it decides the integer sample   */
/* count, which must agree exactly.  Camera = 3x4 row-major pose as in  */
/* nes.proto Camera.matrix (include/base/camera_manager.h:18-19):       */
/* columns 0,1,2 = image right, image down, view direction; column 3 =  */
/* eye position.  Pixel centres, focal length in pixels (horizontal FOV)*/
/* Unit-cube slab clip; n = min(1024, floor((t_far - t_start)/dt)).     */
/* ------------------------------------------------------------------ */
int oracle_ray_setup(const float *M, int W, int H, float focal, int px, int py, float *o,
                     float *d, float *t_start_out) {
  volatile float u = ((float)px + 0.5f - 0.5f * (float)W) / focal;
  volatile float v = ((float)py + 0.5f - 0.5f * (float)H) / focal;
  float dv[3];
  for (int a = 0; a < 3; a++) {
    volatile float p0 = M[a * 4 + 0] * u;
    volatile float p1 = M[a * 4 + 1] * v;
    volatile float s = p0 + p1;
    dv[a] = s + M[a * 4 + 2];
  }
  volatile float q0 = dv[0] * dv[0];
  volatile float q1 = dv[1] * dv[1];
  volatile float q2 = dv[2] * dv[2];
  volatile float n2 = (q0 + q1) + q2;
  float nrm = sqrtf(n2);
  for (int a = 0; a < 3; a++) {
    d[a] = dv[a] / nrm;
    o[a] = M[a * 4 + 3];
  }
  float tn = -INFINITY, tf = INFINITY;
  for (int a = 0; a < 3; a++) {
    volatile float inv = 1.0f / d[a];
    volatile float t0 = (0.0f - o[a]) * inv;
    volatile float t1 = (1.0f - o[a]) * inv;
    tn = fmaxf(tn, fminf(t0, t1));
    tf = fminf(tf, fmaxf(t0, t1));
  }
  float ts = fmaxf(tn, 0.0f);
  *t_start_out = ts;
  if (!(tf > ts)) return 0;
  volatile float span = tf - ts;
  volatile float q = span / OR_DT;
  float fl = floorf(q);
  int n = fl >= (float)OR_MAX_STEPS ? OR_MAX_STEPS : (int)fl;
  return n;
}

/* ------------------------------------------------------------------ */
/* Occupancy grid: 128^3 cells, x-fastest; bit i of word i/32 set when  */
/* the density at the cell centre exceeds the threshold.               */
/* ------------------------------------------------------------------ */
typedef struct {
  const or_scene *s;
  uint32_t *bits;
  double threshold;
  int next_z;
  pthread_mutex_t mu;
} or_occ_job;

static void *or_occ_worker(void *arg) {
  or_occ_job *j = (or_occ_job *)arg;
  for (;;) {
    pthread_mutex_lock(&j->mu);
    int z = j->next_z++;
    pthread_mutex_unlock(&j->mu);
    if (z >= OR_OCC_RES) break;
    for (int y = 0; y < OR_OCC_RES; y++) {
      for (int x = 0; x < OR_OCC_RES; x += 32) {
        uint32_t word = 0;
        for (int b = 0; b < 32; b++) {
          double p[3] = {(x + b + 0.5) / OR_OCC_RES, (y + 0.5) / OR_OCC_RES,
                         (z + 0.5) / OR_OCC_RES};
          if (oracle_density(j->s, p) > j->threshold) word |= 1u << b;
        }
        j->bits[((size_t)z * OR_OCC_RES * OR_OCC_RES + (size_t)y * OR_OCC_RES + x) / 32] = word;
      }
    }
  }
  return NULL;
}

/* bits: 65536 words (256 KiB). threshold <= 0 uses the scene's 0.01. */
void oracle_occupancy(const void *h, double threshold, uint32_t *bits, int nthreads) {
  or_occ_job j;
  j.s = (const or_scene *)h;
  j.bits = bits;
  j.threshold = threshold > 0.0 ? threshold : OR_OCC_THRESHOLD;
  j.next_z = 0;
  pthread_mutex_init(&j.mu, NULL);
  if (nthreads < 1) nthreads = 1;
  pthread_t th[256];
  if (nthreads > 256) nthreads = 256;
  for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, or_occ_worker, &j);
  for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
  pthread_mutex_destroy(&j.mu);
}

static inline int or_occupied(const uint32_t *bits, const double *x) {
  if (!bits) return 1;
  int c[3];
  for (int a = 0; a < 3; a++) {
    int v = (int)floor(x[a] * OR_OCC_RES);
    c[a] = v < 0 ? 0 : (v > OR_OCC_RES - 1 ? OR_OCC_RES - 1 : v);
  }
  size_t i = (size_t)c[0] + (size_t)OR_OCC_RES * ((size_t)c[1] + (size_t)OR_OCC_RES * c[2]);
  return (bits[i >> 5] >> (i & 31)) & 1u;
}

/* ------------------------------------------------------------------ */
/* March + composite one ray in FP64:                                  */
/*   t_i = t_start + (i + 1/2) dt, x_i = o + t_i d clamped to [0,1]^3   */
/*   alpha_i = 1 - exp(-sigma_i dt), w_i = T_i alpha_i,                 */
/*   rgb = sum w_i c_i, depth = sum w_i t_i, T_{i+1} = T_i (1-alpha_i), */
/*   stop after the sample that takes T below 1e-4.  No background.     */
/* Returns the number of samples evaluated (occupied, before stop).     */
/* ------------------------------------------------------------------ */
int oracle_march_ray(const void *h, const uint32_t *occ, const float *of, const float *df,
                     float t_start, int n, double *rgb, double *depth, double *trans) {
  const double dt = (double)OR_DT;
  double o[3] = {of[0], of[1], of[2]}, d[3] = {df[0], df[1], df[2]};
  double T = 1.0, acc[3] = {0, 0, 0}, dep = 0.0;
  int evaluated = 0;
  for (int i = 0; i < n; i++) {
    double t = (double)t_start + ((double)i + 0.5) * dt;
    double x[3];
    for (int a = 0; a < 3; a++) {
      double v = o[a] + t * d[a];
      x[a] = v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
    }
    if (!or_occupied(occ, x)) continue;
    double sigma, c[3];
    oracle_query(h, x, d, &sigma, c);
    evaluated++;
    double alpha = -expm1(-sigma * dt);
    double w = T * alpha;
    for (int a = 0; a < 3; a++) acc[a] += w * c[a];
    dep += w * t;
    T *= 1.0 - alpha;
    if (T < OR_T_STOP) break;
  }
  for (int a = 0; a < 3; a++) rgb[a] = acc[a];
  *depth = dep;
  if (trans) *trans = T;
  return evaluated;
}

typedef struct {
  const or_scene *s;
  const uint32_t *occ;
  const float *M;
  int W, H;
  float focal;
  const int32_t *pix; /* pixel indices (y*W+x) or NULL for all */
  long npix;
  double *rgb, *depth;
  long next;
  long long samples;
  pthread_mutex_t mu;
} or_render_job;

static void *or_render_worker(void *arg) {
  or_render_job *j = (or_render_job *)arg;
  long long local_samples = 0;
  for (;;) {
    pthread_mutex_lock(&j->mu);
    long b = j->next;
    j->next += 64;
    pthread_mutex_unlock(&j->mu);
    if (b >= j->npix) break;
    long e = b + 64 < j->npix ? b + 64 : j->npix;
    for (long k = b; k < e; k++) {
      long p = j->pix ? (long)j->pix[k] : k;
      int px = (int)(p % j->W), py = (int)(p / j->W);
      float o[3], d[3], ts;
      int n = oracle_ray_setup(j->M, j->W, j->H, j->focal, px, py, o, d, &ts);
      double rgb[3] = {0, 0, 0}, dep = 0.0;
      if (n > 0) local_samples += oracle_march_ray(j->s, j->occ, o, d, ts, n, rgb, &dep, NULL);
      for (int a = 0; a < 3; a++) j->rgb[k * 3 + a] = rgb[a];
      j->depth[k] = dep;
    }
  }
  pthread_mutex_lock(&j->mu);
  j->samples += local_samples;
  pthread_mutex_unlock(&j->mu);
  return NULL;
}

/* Render the listed pixels (or all W*H when pix == NULL) of one view.
 * rgb: npix*3 doubles, depth: npix doubles.  occ may be NULL (all cells
 * occupied).  Returns the number of field evaluations. */
long long oracle_render(const void *h, const uint32_t *occ, const float *M, int W, int H,
                        float focal, const int32_t *pix, long npix, double *rgb, double *depth,
                        int nthreads) {
  or_render_job j;
  j.s = (const or_scene *)h;
  j.occ = occ;
  j.M = M;
  j.W = W;
  j.H = H;
  j.focal = focal;
  j.pix = pix;
  j.npix = pix ? npix : (long)W * H;
  j.rgb = rgb;
  j.depth = depth;
  j.next = 0;
  j.samples = 0;
  pthread_mutex_init(&j.mu, NULL);
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, or_render_worker, &j);
  for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
  pthread_mutex_destroy(&j.mu);
  return j.samples;
}

/* ------------------------------------------------------------------ */
/* Frame glue: BT.601 studio range, 16 fractional bits.                */
/*   Y  = 16  + (219/255)(0.299 R + 0.587 G + 0.114 B)                   */
/*   Cb = 128 + (224/255)(B - Y')/1.772,  Cr = 128 + (224/255)(R - Y')/1.402 */
/* Luma per pixel; chroma from the sum of the 2x2 block (edge pixels    */
/* replicated for odd sizes), i.e. the block average.  Luma            */
/* coefficients are rounded with their sum pinned to round(219/255*2^16);*/
/* each chroma row is adjusted to sum to zero so grey maps to 128.     */
/* ------------------------------------------------------------------ */
enum {
  OR_YR = 16829, OR_YG = 33039, OR_YB = 6416,
  OR_UR = -9714, OR_UG = -19071, OR_UB = 28785,
  OR_VR = 28784, OR_VG = -24103, OR_VB = -4681
};

static inline uint8_t or_clamp8(int32_t v) { return (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v)); }

void oracle_rgb24_to_yuv420p(const uint8_t *rgb, int w, int h, int rgb_ls, uint8_t *y, uint8_t *u,
                             uint8_t *v, const int *ls) {
  for (int r = 0; r < h; r++)
    for (int c = 0; c < w; c++) {
      const uint8_t *p = rgb + (size_t)r * rgb_ls + (size_t)c * 3;
      int32_t s = OR_YR * p[0] + OR_YG * p[1] + OR_YB * p[2] + (16 << 16) + (1 << 15);
      y[(size_t)r * ls[0] + c] = or_clamp8(s >> 16);
    }
  int cw = (w + 1) / 2, ch = (h + 1) / 2;
  for (int r = 0; r < ch; r++)
    for (int c = 0; c < cw; c++) {
      int32_t sr = 0, sg = 0, sb = 0;
      for (int dy = 0; dy < 2; dy++)
        for (int dx = 0; dx < 2; dx++) {
          int rr = 2 * r + dy, cc = 2 * c + dx;
          if (rr > h - 1) rr = h - 1;
          if (cc > w - 1) cc = w - 1;
          const uint8_t *p = rgb + (size_t)rr * rgb_ls + (size_t)cc * 3;
          sr += p[0];
          sg += p[1];
          sb += p[2];
        }
      int32_t cb = OR_UR * sr + OR_UG * sg + OR_UB * sb + (128 << 18) + (1 << 17);
      int32_t cr = OR_VR * sr + OR_VG * sg + OR_VB * sb + (128 << 18) + (1 << 17);
      u[(size_t)r * ls[1] + c] = or_clamp8(cb >> 18);
      v[(size_t)r * ls[2] + c] = or_clamp8(cr >> 18);
    }
}

void oracle_gray8_to_yuv420p(const uint8_t *g, int w, int h, int g_ls, uint8_t *y, uint8_t *u,
                             uint8_t *v, const int *ls) {
  const int32_t ys = OR_YR + OR_YG + OR_YB;
  for (int r = 0; r < h; r++)
    for (int c = 0; c < w; c++) {
      int32_t s = ys * g[(size_t)r * g_ls + c] + (16 << 16) + (1 << 15);
      y[(size_t)r * ls[0] + c] = or_clamp8(s >> 16);
    }
  int cw = (w + 1) / 2, ch = (h + 1) / 2;
  for (int r = 0; r < ch; r++)
    for (int c = 0; c < cw; c++) {
      u[(size_t)r * ls[1] + c] = 128;
      v[(size_t)r * ls[2] + c] = 128;
    }
}

/* FP32 scene units (metres) -> uint16 millimetres: round half up of d*1000
 * in FP32, NaN and negatives to 0, saturating at 65535. */
void oracle_depth_pack_u16mm(const float *d, long n, uint16_t *out) {
  for (long i = 0; i < n; i++) {
    volatile float mm = d[i] * 1000.0f;
    uint16_t q;
    if (!(mm >= 0.0f))
      q = 0;
    else if (mm >= 65535.0f)
      q = 65535;
    else {
      volatile float r = mm + 0.5f;
      q = (uint16_t)(uint32_t)r;
    }
    out[i] = q;
  }
}

/* FP32 depth -> GRAY8 (the reference's depth plane, src/server.cpp:194):
 * round(clamp(d / dmax, 0, 1) * 255), in FP32. */
void oracle_depth_to_gray8(const float *d, long n, float dmax, uint8_t *out) {
  for (long i = 0; i < n; i++) {
    volatile float q = d[i] / dmax;
    float c = q > 0.0f ? (q < 1.0f ? q : 1.0f) : 0.0f;
    volatile float s = c * 255.0f;
    volatile float r = s + 0.5f;
    out[i] = (uint8_t)(uint32_t)r;
  }
}

/* FP32 RGB in [0,1] -> RGB24: round(clamp(x,0,1) * 255), in FP32. */
void oracle_rgb_to_rgb24(const float *rgb, long n, uint8_t *out) {
  for (long i = 0; i < n; i++) {
    float x = rgb[i];
    float c = x > 0.0f ? (x < 1.0f ? x : 1.0f) : 0.0f;
    volatile float s = c * 255.0f;
    volatile float r = s + 0.5f;
    out[i] = (uint8_t)(uint32_t)r;
  }
}

/* ------------------------------------------------------------------ */
/* Debug text overlay (RenderTextContext::render_string_to_frame,      */
/* src/base/video/render_text.cc:35-111): five anchors with margin 50  */
/* and a 300x100 box, '\n' = anchor column and 20 px down, covered      */
/* pixels set to white, clipped.  Glyphs: 5x7 dot matrix drawn at 2x,   */
/* 12 px advance, bottom row on the pen's baseline.                     */
/* ------------------------------------------------------------------ */
static const struct {
  char c;
  unsigned char r[7];
} OR_GLYPHS[] = {
    {'0', {14, 17, 19, 21, 25, 17, 14}}, {'1', {4, 12, 4, 4, 4, 4, 14}},     {'2', {14, 17, 1, 2, 4, 8, 31}},
    {'3', {30, 1, 1, 14, 1, 1, 30}},     {'4', {2, 6, 10, 18, 31, 2, 2}},    {'5', {31, 16, 30, 1, 1, 17, 14}},
    {'6', {6, 8, 16, 30, 17, 17, 14}},   {'7', {31, 1, 2, 4, 8, 8, 8}},      {'8', {14, 17, 17, 14, 17, 17, 14}},
    {'9', {14, 17, 17, 15, 1, 2, 12}},   {'+', {0, 4, 4, 31, 4, 4, 0}},      {'-', {0, 0, 0, 31, 0, 0, 0}},
    {'.', {0, 0, 0, 0, 0, 12, 12}},      {':', {0, 12, 12, 0, 12, 12, 0}},   {'=', {0, 0, 31, 0, 31, 0, 0}},
    {'a', {0, 0, 14, 1, 15, 17, 15}},    {'b', {16, 16, 22, 25, 17, 17, 30}}, {'c', {0, 0, 14, 16, 16, 17, 14}},
    {'d', {1, 1, 13, 19, 17, 17, 15}},   {'e', {0, 0, 14, 17, 31, 16, 14}},  {'f', {6, 9, 8, 28, 8, 8, 8}},
    {'g', {0, 15, 17, 17, 15, 1, 14}},   {'h', {16, 16, 22, 25, 17, 17, 17}}, {'i', {4, 0, 12, 4, 4, 4, 14}},
    {'j', {2, 0, 6, 2, 2, 18, 12}},      {'k', {16, 16, 18, 20, 24, 20, 18}}, {'l', {12, 4, 4, 4, 4, 4, 14}},
    {'m', {0, 0, 26, 21, 21, 17, 17}},   {'n', {0, 0, 22, 25, 17, 17, 17}},  {'o', {0, 0, 14, 17, 17, 17, 14}},
    {'p', {0, 0, 30, 17, 30, 16, 16}},   {'q', {0, 0, 13, 19, 15, 1, 1}},    {'r', {0, 0, 22, 25, 16, 16, 16}},
    {'s', {0, 0, 14, 16, 14, 1, 30}},    {'t', {8, 8, 28, 8, 8, 9, 6}},      {'u', {0, 0, 17, 17, 17, 19, 13}},
    {'v', {0, 0, 17, 17, 17, 10, 4}},    {'w', {0, 0, 17, 17, 21, 21, 10}},  {'x', {0, 0, 17, 10, 4, 10, 17}},
    {'y', {0, 0, 17, 17, 15, 1, 14}},    {'z', {0, 0, 31, 2, 4, 8, 31}},
};

static const unsigned char *or_glyph(char c) {
  for (size_t i = 0; i < sizeof(OR_GLYPHS) / sizeof(OR_GLYPHS[0]); i++)
    if (OR_GLYPHS[i].c == c) return OR_GLYPHS[i].r;
  return NULL;
}

void oracle_overlay_text(uint8_t *rgb, int w, int h, int ls, const char *text, int anchor) {
  const int x_box = 300, y_box = 100, margin = 50;
  int pen_x = margin, pen_y = margin;
  if (anchor == 1) { pen_x = margin; pen_y = h - y_box + margin; }
  else if (anchor == 2) { pen_x = w - x_box + margin; pen_y = margin; }
  else if (anchor == 3) { pen_x = w - x_box + margin; pen_y = h - y_box + margin; }
  else if (anchor == 4) { pen_x = w / 2 - x_box; pen_y = h / 2 - y_box; }
  const int x0 = pen_x;
  for (const char *c = text; *c; c++) {
    if (*c == '\n') {
      pen_x = x0;
      pen_y += 20;
      continue;
    }
    const unsigned char *g = or_glyph(*c);
    if (g) {
      for (int py = 0; py < 14; py++)
        for (int px = 0; px < 10; px++) {
          if (!((g[py / 2] >> (4 - px / 2)) & 1)) continue;
          int X = pen_x + px, Y = pen_y - 14 + py;
          if (X < 0 || Y < 0 || X >= w || Y >= h) continue;
          uint8_t *q = rgb + (size_t)Y * ls + (size_t)X * 3;
          q[0] = q[1] = q[2] = 255;
        }
    }
    pen_x += 12;
  }
}

/* ------------------------------------------------------------------ */
/* Training loss and its gradient, FP64, by reverse-mode sweeps (the    */
/* checker of the product's nes_trainer_grad).  Per ray r of the batch  */
/* of n: L_r = |C - C*|^2 + depth_w (D - D*)^2 with C, D from           */
/* oracle_march_ray's compositing; L = mean of L_r.  The compositing    */
/* adjoint runs backwards over the ray's samples carrying A = dL/dT_k:  */
/*   g_w = dL/dw_k = g_C . c_k + g_D t_k,                               */
/*   dL/dsigma_k = dt T_{k+1} (g_w - A_{k+1}),  dL/dc_k = g_C w_k,      */
/*   A_k = g_w alpha_k + A_{k+1} (1 - alpha_k),  A_K = 0;               */
/* then each sample backpropagates through both MLPs (ReLU derivative   */
/* taken as 0 at 0) and the trilinear hash-grid lookup.                 */
/* fp32_positions: sample t and x by the CUDA kernels' FP32 fused       */
/* multiply-adds (t = fma(i + 1/2, dt, t_start), x = clamp(fma(t, d, o)))*/
/* and grid cells from x*N rounded to FP32, instead of FP64, to isolate */
/* the gradient arithmetic from the FP32 rounding of sample positions.  */
/* g_table: 16*T*2 doubles, g_w: 9408 doubles (dw1|dw2|cw1|cw2|cw3),    */
/* both accumulated (+=); both NULL: loss only.  Returns L.            */
/* ------------------------------------------------------------------ */
/* fp32_cells: the cell coordinate x*N rounded to FP32 first, as the CUDA
 * kernels compute it (the rounding can carry x*N up to the next integer). */
static void or_encode_corners(const or_scene *s, const double *x, int fp32_cells, double *feat,
                              uint32_t idx[OR_LEVELS][8], double wts[OR_LEVELS][8]) {
  for (int l = 0; l < OR_LEVELS; l++) {
    int N = OR_RES[l];
    double f[3];
    uint32_t i0[3];
    for (int a = 0; a < 3; a++) {
      double p = fp32_cells ? (double)(float)(x[a] * (double)N) : x[a] * (double)N;
      double fl = floor(p);
      if (fl < 0.0) fl = 0.0;
      if (fl > (double)(N - 1)) fl = (double)(N - 1);
      i0[a] = (uint32_t)fl;
      f[a] = p - fl;
    }
    const float *tab = s->table + (size_t)l * s->T * OR_FEATS;
    double a0 = 0.0, a1 = 0.0;
    for (int c = 0; c < 8; c++) {
      int dx = c & 1, dy = (c >> 1) & 1, dz = (c >> 2) & 1;
      wts[l][c] = (dx ? f[0] : 1.0 - f[0]) * (dy ? f[1] : 1.0 - f[1]) * (dz ? f[2] : 1.0 - f[2]);
      idx[l][c] = oracle_grid_index((uint32_t)l, s->T, i0[0] + dx, i0[1] + dy, i0[2] + dz);
      a0 += wts[l][c] * (double)tab[(size_t)idx[l][c] * 2 + 0];
      a1 += wts[l][c] * (double)tab[(size_t)idx[l][c] * 2 + 1];
    }
    feat[2 * l] = a0;
    feat[2 * l + 1] = a1;
  }
}

static void or_query_cells(const or_scene *s, const double *x, const double *d, int fp32_cells,
                           double *sigma, double *rgb) {
  double enc[OR_ENC], h1[OR_HID], out[OR_DOUT], cin[OR_CIN], g1[OR_HID], g2[OR_HID];
  uint32_t idx[OR_LEVELS][8];
  double wts[OR_LEVELS][8];
  or_encode_corners(s, x, fp32_cells, enc, idx, wts);
  or_density(s, enc, h1, out);
  *sigma = exp(out[0] - 1.0);
  oracle_sh16(d, cin);
  for (int i = 0; i < 15; i++) cin[16 + i] = out[1 + i];
  cin[31] = 0.0;
  or_colour(s, cin, g1, g2, rgb);
}

static void or_sample_backward(const or_scene *s, const double *x, const double *d, int fp32_cells,
                               double dsigma, const double *dc, double *g_table, double *g_w) {
  double enc[OR_ENC], h1[OR_HID], out[OR_DOUT], cin[OR_CIN], g1[OR_HID], g2[OR_HID], rgb[3];
  uint32_t idx[OR_LEVELS][8];
  double wts[OR_LEVELS][8];
  or_encode_corners(s, x, fp32_cells, enc, idx, wts);
  or_density(s, enc, h1, out);
  double sigma = exp(out[0] - 1.0);
  oracle_sh16(d, cin);
  for (int i = 0; i < 15; i++) cin[16 + i] = out[1 + i];
  cin[31] = 0.0;
  or_colour(s, cin, g1, g2, rgb);
  double *gdw1 = g_w, *gdw2 = g_w + 2048, *gcw1 = g_w + 3072, *gcw2 = g_w + 5120, *gcw3 = g_w + 9216;
  double dl[3], dg2[OR_HID], dg1[OR_HID], dcin[OR_CIN], dout[OR_DOUT], dh1[OR_HID], denc[OR_ENC];
  for (int c = 0; c < 3; c++) dl[c] = dc[c] * rgb[c] * (1.0 - rgb[c]);
  for (int c = 0; c < 3; c++)
    for (int j = 0; j < OR_HID; j++) gcw3[c * OR_HID + j] += dl[c] * g2[j];
  for (int j = 0; j < OR_HID; j++) {
    double a = 0.0;
    for (int c = 0; c < 3; c++) a += (double)s->cw3[c * OR_HID + j] * dl[c];
    dg2[j] = g2[j] > 0.0 ? a : 0.0;
  }
  for (int j = 0; j < OR_HID; j++)
    for (int k = 0; k < OR_HID; k++) gcw2[j * OR_HID + k] += dg2[j] * g1[k];
  for (int k = 0; k < OR_HID; k++) {
    double a = 0.0;
    for (int j = 0; j < OR_HID; j++) a += (double)s->cw2[j * OR_HID + k] * dg2[j];
    dg1[k] = g1[k] > 0.0 ? a : 0.0;
  }
  for (int j = 0; j < OR_HID; j++)
    for (int k = 0; k < OR_CIN; k++) gcw1[j * OR_CIN + k] += dg1[j] * cin[k];
  for (int k = 0; k < OR_CIN; k++) {
    double a = 0.0;
    for (int j = 0; j < OR_HID; j++) a += (double)s->cw1[j * OR_CIN + k] * dg1[j];
    dcin[k] = a;
  }
  dout[0] = dsigma * sigma;
  for (int i = 0; i < 15; i++) dout[1 + i] = dcin[16 + i];
  for (int m = 0; m < OR_DOUT; m++)
    for (int j = 0; j < OR_HID; j++) gdw2[m * OR_HID + j] += dout[m] * h1[j];
  for (int j = 0; j < OR_HID; j++) {
    double a = 0.0;
    for (int m = 0; m < OR_DOUT; m++) a += (double)s->dw2[m * OR_HID + j] * dout[m];
    dh1[j] = h1[j] > 0.0 ? a : 0.0;
  }
  for (int j = 0; j < OR_HID; j++)
    for (int k = 0; k < OR_ENC; k++) gdw1[j * OR_ENC + k] += dh1[j] * enc[k];
  for (int k = 0; k < OR_ENC; k++) {
    double a = 0.0;
    for (int j = 0; j < OR_HID; j++) a += (double)s->dw1[j * OR_ENC + k] * dh1[j];
    denc[k] = a;
  }
  for (int l = 0; l < OR_LEVELS; l++) {
    double *gt = g_table + (size_t)l * s->T * OR_FEATS;
    for (int c = 0; c < 8; c++) {
      gt[(size_t)idx[l][c] * 2 + 0] += wts[l][c] * denc[2 * l + 0];
      gt[(size_t)idx[l][c] * 2 + 1] += wts[l][c] * denc[2 * l + 1];
    }
  }
}

double oracle_train_loss_grad(const void *h, const uint32_t *occ, const float *o, const float *d,
                              const float *ts, const int *nsteps, int n, const double *target,
                              double depth_w, int fp32_positions, double *g_table, double *g_w) {
  const or_scene *s = (const or_scene *)h;
  const double dt = (double)OR_DT;
  double loss = 0.0;
  double *xs = (double *)malloc(sizeof(double) * OR_MAX_STEPS * 7); /* x[3], t, sigma, alpha, T_k */
  double *cs = (double *)malloc(sizeof(double) * OR_MAX_STEPS * 3);
  if (!xs || !cs) {
    free(xs);
    free(cs);
    return NAN;
  }
  for (int r = 0; r < n; r++) {
    double od[3] = {o[3 * r], o[3 * r + 1], o[3 * r + 2]}, dd[3] = {d[3 * r], d[3 * r + 1], d[3 * r + 2]};
    double T = 1.0, C[3] = {0, 0, 0}, D = 0.0;
    int K = 0;
    for (int i = 0; i < nsteps[r]; i++) {
      double t, x[3];
      if (fp32_positions) { /* the CUDA kernels' FP32 fused multiply-adds */
        float tf = fmaf((float)i + 0.5f, OR_DT, ts[r]);
        t = tf;
        for (int a = 0; a < 3; a++) {
          float v = fmaf(tf, d[3 * r + a], o[3 * r + a]);
          x[a] = v < 0.0f ? 0.0 : (v > 1.0f ? 1.0 : (double)v);
        }
      } else {
        t = (double)ts[r] + ((double)i + 0.5) * dt;
        for (int a = 0; a < 3; a++) {
          double v = od[a] + t * dd[a];
          x[a] = v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
        }
      }
      if (!or_occupied(occ, x)) continue;
      double sigma, c[3];
      or_query_cells(s, x, dd, fp32_positions, &sigma, c);
      double alpha = -expm1(-sigma * dt);
      double w = T * alpha;
      double *q = xs + 7 * K;
      q[0] = x[0]; q[1] = x[1]; q[2] = x[2]; q[3] = t; q[4] = sigma; q[5] = alpha; q[6] = T;
      cs[3 * K] = c[0]; cs[3 * K + 1] = c[1]; cs[3 * K + 2] = c[2];
      K++;
      for (int a = 0; a < 3; a++) C[a] += w * c[a];
      D += w * t;
      T *= 1.0 - alpha;
      if (T < OR_T_STOP) break;
    }
    const double *tg = target + 4 * r;
    double e[3] = {C[0] - tg[0], C[1] - tg[1], C[2] - tg[2]}, ed = D - tg[3];
    loss += (e[0] * e[0] + e[1] * e[1] + e[2] * e[2] + depth_w * ed * ed) / n;
    double gC[3] = {2.0 * e[0] / n, 2.0 * e[1] / n, 2.0 * e[2] / n}, gD = 2.0 * depth_w * ed / n;
    double A = 0.0;
    for (int k = K - 1; k >= 0; k--) {
      const double *q = xs + 7 * k, *c = cs + 3 * k;
      double alpha = q[5], Tk = q[6], w = Tk * alpha;
      double gw = gC[0] * c[0] + gC[1] * c[1] + gC[2] * c[2] + gD * q[3];
      double dsigma = dt * Tk * (1.0 - alpha) * (gw - A);
      double dc[3] = {gC[0] * w, gC[1] * w, gC[2] * w};
      if (g_table && g_w) or_sample_backward(s, q, dd, fp32_positions, dsigma, dc, g_table, g_w);
      A = gw * alpha + A * (1.0 - alpha);
    }
  }
  free(xs);
  free(cs);
  return loss;
}

/* ------------------------------------------------------------------ */
/* Plain FP32 CPU render: the same scene, march and compositing in     */
/* single precision, pthreads over host cores.  A CPU speed baseline    */
/* (the FP32 counterpart of the GPU plain path), not a checker.         */
/* ------------------------------------------------------------------ */
static void or_query_f32(const or_scene *s, const float *x, const float *sh, float *sigma, float *rgb) {
  float enc[OR_ENC], h1[OR_HID], out[OR_DOUT], cin[OR_CIN], g1[OR_HID];
  for (int l = 0; l < OR_LEVELS; l++) {
    int N = OR_RES[l];
    float f[3];
    uint32_t i0[3];
    for (int a = 0; a < 3; a++) {
      float p = x[a] * (float)N;
      float fl = floorf(p);
      if (fl < 0.0f) fl = 0.0f;
      if (fl > (float)(N - 1)) fl = (float)(N - 1);
      i0[a] = (uint32_t)fl;
      f[a] = p - fl;
    }
    const float *tab = s->table + (size_t)l * s->T * OR_FEATS;
    float a0 = 0.0f, a1 = 0.0f;
    for (int c = 0; c < 8; c++) {
      int dx = c & 1, dy = (c >> 1) & 1, dz = (c >> 2) & 1;
      float w = (dx ? f[0] : 1.0f - f[0]) * (dy ? f[1] : 1.0f - f[1]) * (dz ? f[2] : 1.0f - f[2]);
      uint32_t idx = oracle_grid_index((uint32_t)l, s->T, i0[0] + dx, i0[1] + dy, i0[2] + dz);
      a0 += w * tab[(size_t)idx * 2];
      a1 += w * tab[(size_t)idx * 2 + 1];
    }
    enc[2 * l] = a0;
    enc[2 * l + 1] = a1;
  }
  for (int m = 0; m < OR_DOUT; m++) out[m] = 0.0f;
  for (int j = 0; j < OR_HID; j++) {
    float a = 0.0f;
    for (int k = 0; k < OR_ENC; k++) a += s->dw1[j * OR_ENC + k] * enc[k];
    h1[j] = a > 0.0f ? a : 0.0f;
  }
  for (int m = 0; m < OR_DOUT; m++) {
    float a = 0.0f;
    for (int j = 0; j < OR_HID; j++) a += s->dw2[m * OR_HID + j] * h1[j];
    out[m] = a;
  }
  *sigma = expf(out[0] - 1.0f);
  for (int k = 0; k < 16; k++) cin[k] = sh[k];
  for (int k = 0; k < 15; k++) cin[16 + k] = out[1 + k];
  cin[31] = 0.0f;
  for (int j = 0; j < OR_HID; j++) {
    float a = 0.0f;
    for (int k = 0; k < OR_CIN; k++) a += s->cw1[j * OR_CIN + k] * cin[k];
    g1[j] = a > 0.0f ? a : 0.0f;
  }
  float lg[3] = {0.0f, 0.0f, 0.0f};
  for (int j = 0; j < OR_HID; j++) {
    float a = 0.0f;
    for (int k = 0; k < OR_HID; k++) a += s->cw2[j * OR_HID + k] * g1[k];
    a = a > 0.0f ? a : 0.0f;
    for (int c = 0; c < 3; c++) lg[c] += s->cw3[c * OR_HID + j] * a;
  }
  for (int c = 0; c < 3; c++) rgb[c] = 1.0f / (1.0f + expf(-lg[c]));
}

typedef struct {
  const or_scene *s;
  const uint32_t *occ;
  const float *M;
  int W, H;
  float focal;
  const int32_t *pix;
  long npix;
  float *rgb, *depth;
  long next;
  long long samples;
  pthread_mutex_t mu;
} or_render32_job;

static void *or_render32_worker(void *arg) {
  or_render32_job *j = (or_render32_job *)arg;
  long long local = 0;
  for (;;) {
    pthread_mutex_lock(&j->mu);
    long b = j->next;
    j->next += 64;
    pthread_mutex_unlock(&j->mu);
    if (b >= j->npix) break;
    long e = b + 64 < j->npix ? b + 64 : j->npix;
    for (long k = b; k < e; k++) {
      long p = j->pix ? (long)j->pix[k] : k;
      float o[3], d[3], ts;
      int n = oracle_ray_setup(j->M, j->W, j->H, j->focal, (int)(p % j->W), (int)(p / j->W), o, d, &ts);
      float C[3] = {0.0f, 0.0f, 0.0f}, D = 0.0f, T = 1.0f;
      double dd[3] = {d[0], d[1], d[2]}, shd[16];
      float sh[16];
      oracle_sh16(dd, shd);
      for (int i = 0; i < 16; i++) sh[i] = (float)shd[i];
      for (int i = 0; i < n; i++) {
        float t = ts + ((float)i + 0.5f) * OR_DT;
        float x[3];
        double xd[3];
        for (int a = 0; a < 3; a++) {
          float v = o[a] + t * d[a];
          x[a] = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
          xd[a] = x[a];
        }
        if (!or_occupied(j->occ, xd)) continue;
        float sigma, c[3];
        or_query_f32(j->s, x, sh, &sigma, c);
        local++;
        float alpha = -expm1f(-sigma * OR_DT), w = T * alpha;
        for (int a = 0; a < 3; a++) C[a] += w * c[a];
        D += w * t;
        T -= w;
        if (T < (float)OR_T_STOP) break;
      }
      for (int a = 0; a < 3; a++) j->rgb[k * 3 + a] = C[a];
      j->depth[k] = D;
    }
  }
  pthread_mutex_lock(&j->mu);
  j->samples += local;
  pthread_mutex_unlock(&j->mu);
  return NULL;
}

/* FP32 render of the listed pixels (or all W*H); rgb npix*3, depth npix
 * floats.  Returns the number of field evaluations. */
long long oracle_render_f32(const void *h, const uint32_t *occ, const float *M, int W, int H, float focal,
                            const int32_t *pix, long npix, float *rgb, float *depth, int nthreads) {
  or_render32_job j;
  j.s = (const or_scene *)h;
  j.occ = occ;
  j.M = M;
  j.W = W;
  j.H = H;
  j.focal = focal;
  j.pix = pix;
  j.npix = pix ? npix : (long)W * H;
  j.rgb = rgb;
  j.depth = depth;
  j.next = 0;
  j.samples = 0;
  pthread_mutex_init(&j.mu, NULL);
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, or_render32_worker, &j);
  for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
  pthread_mutex_destroy(&j.mu);
  return j.samples;
}
