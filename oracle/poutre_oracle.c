/*
 * poutre_oracle.c -- CPU restatement of poutre2's morphology + geodesy hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: it is built into
 * oracle/_build/libpoutre_oracle.so and loaded by the test-suite, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  The product
 * library (poutre2_gb300/csrc) never links, loads or calls it.
 *
 * Every routine restates the reference algorithm it cites (paths are relative
 * to the poutre2 source tree) in plain C.  Parity is pinned by the reference's
 * own known-answer tests (tests/golden/reference_kats.json, extracted from the
 * test/low_level_morpho and test/geodesy Catch2 files) and, where the reference
 * compiles, by direct comparison with it on random inputs (oracle/ref).
 *
 * Conventions
 *   - images are dense row-major, last dimension fastest (array_view.hpp:908-912);
 *     a rank-r image of reference shape {d0..dr-1} is handled internally as
 *     (nz, ny, nx) = (1,1,d0) | (1,d0,d1) | (d0,d1,d2).
 *   - structuring-element offsets are (dz, dy, dx) triples in the same order.
 *   - ptype codes are poutre::PType values (types.hpp:517-526) plus 128 for
 *     uint16, which the reference does not have.
 *   - return value: 0 on success, negative on an argument the reference rejects.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

enum { PT_U8 = 4, PT_I32 = 8, PT_F32 = 16, PT_I64 = 32, PT_F64 = 64, PT_U16 = 128 };

/* Common_NL_SE, se_types_and_tags.hpp:45-57 */
enum {
  SE_UNDEF = 0, SE_SEGX1D, SE_SQUARE2D, SE_CROSS2D, SE_SEGX2D, SE_SEGY2D,
  SE_SEGX3D, SE_SEGY3D, SE_SEGZ3D, SE_CROSS3D, SE_SQUARE3D
};

typedef struct { int dz, dy, dx; } off3;

/* ------------------------------------------------------------------------- */
/* Structuring-element tables.                                                */
/* Full lists (centre first): neighbor_list_static_se_t.hpp:38-431 and        */
/* src/structuring_element/predefined_nl_se.cpp:19-92.                        */
/* Upper/lower raster halves: split_coordinates_upper_lower() of the same     */
/* traits (used by the reconstruction scans).                                 */
/* ------------------------------------------------------------------------- */
static const off3 T_SEGX1D[] = {{0, 0, 0}, {0, 0, -1}, {0, 0, 1}};
static const off3 T_SEGX2D[] = {{0, 0, 0}, {0, 0, -1}, {0, 0, 1}};
static const off3 T_SEGY2D[] = {{0, 0, 0}, {0, -1, 0}, {0, 1, 0}};
static const off3 T_SQUARE2D[] = {{0, 0, 0}, {0, -1, -1}, {0, 0, -1}, {0, 1, -1}, {0, -1, 0},
                                  {0, 1, 0}, {0, -1, 1}, {0, 0, 1}, {0, 1, 1}};
static const off3 T_CROSS2D[] = {{0, 0, 0}, {0, 0, -1}, {0, -1, 0}, {0, 1, 0}, {0, 0, 1}};
static const off3 T_SEGX3D[] = {{0, 0, 0}, {0, 0, -1}, {0, 0, 1}};
static const off3 T_SEGY3D[] = {{0, 0, 0}, {0, -1, 0}, {0, 1, 0}};
static const off3 T_SEGZ3D[] = {{0, 0, 0}, {-1, 0, 0}, {1, 0, 0}};
static const off3 T_CROSS3D[] = {{0, 0, 0}, {0, 0, -1}, {0, -1, 0}, {-1, 0, 0},
                                 {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
static off3 T_SQUARE3D[27];

/* upper / lower halves (reconstruction), same traits */
static const off3 U_SEGX1D[] = {{0, 0, -1}};
static const off3 L_SEGX1D[] = {{0, 0, 1}};
static const off3 U_SQUARE2D[] = {{0, -1, -1}, {0, -1, 0}, {0, -1, 1}, {0, 0, -1}};
static const off3 L_SQUARE2D[] = {{0, 0, 1}, {0, 1, -1}, {0, 1, 0}, {0, 1, 1}};
static const off3 U_CROSS2D[] = {{0, -1, 0}, {0, 0, -1}};
static const off3 L_CROSS2D[] = {{0, 1, 0}, {0, 0, 1}};
static const off3 U_CROSS3D[] = {{0, 0, -1}, {0, -1, 0}, {-1, 0, 0}};
static const off3 L_CROSS3D[] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
/* SESquare3D halves as written in neighbor_list_static_se_t.hpp:398-429 (not
 * consistent with raster order; reproduced as-is). */
static const off3 U_SQUARE3D[] = {{1, 0, 0}, {-1, 1, 0}, {0, 1, 0}, {1, 1, 0}, {-1, -1, 1},
                                  {0, -1, 1}, {1, -1, 1}, {-1, 0, 1}, {0, 0, 1}, {1, 0, 1},
                                  {-1, 1, 1}, {0, 1, 1}, {1, 1, 1}};
static const off3 L_SQUARE3D[] = {{-1, -1, -1}, {0, -1, -1}, {1, -1, -1}, {-1, 0, -1}, {0, 0, -1},
                                  {1, 0, -1}, {-1, 1, -1}, {0, 1, -1}, {1, 1, -1}, {-1, -1, 0},
                                  {0, -1, 0}, {1, -1, 0}, {-1, 0, 0}};

static void init_square3d(void) {
  /* centre first, then d2-major, d1, d0 as in the static traits (:360-389) */
  int k = 0;
  T_SQUARE3D[k++] = (off3){0, 0, 0};
  for (int c = -1; c <= 1; ++c)
    for (int b = -1; b <= 1; ++b)
      for (int a = -1; a <= 1; ++a) {
        if (a == 0 && b == 0 && c == 0) continue;
        T_SQUARE3D[k++] = (off3){a, b, c};
      }
}

static int se_rank(int se) {
  switch (se) {
    case SE_SEGX1D: return 1;
    case SE_SQUARE2D: case SE_CROSS2D: case SE_SEGX2D: case SE_SEGY2D: return 2;
    case SE_SEGX3D: case SE_SEGY3D: case SE_SEGZ3D: case SE_CROSS3D: case SE_SQUARE3D: return 3;
    default: return 0;
  }
}

static int se_table(int se, const off3 **tab) {
  init_square3d();
  switch (se) {
    case SE_SEGX1D: *tab = T_SEGX1D; return 3;
    case SE_SQUARE2D: *tab = T_SQUARE2D; return 9;
    case SE_CROSS2D: *tab = T_CROSS2D; return 5;
    case SE_SEGX2D: *tab = T_SEGX2D; return 3;
    case SE_SEGY2D: *tab = T_SEGY2D; return 3;
    case SE_SEGX3D: *tab = T_SEGX3D; return 3;
    case SE_SEGY3D: *tab = T_SEGY3D; return 3;
    case SE_SEGZ3D: *tab = T_SEGZ3D; return 3;
    case SE_CROSS3D: *tab = T_CROSS3D; return 7;
    case SE_SQUARE3D: *tab = T_SQUARE3D; return 27;
    default: return -1;
  }
}

static int se_halves(int se, const off3 **up, int *nu, const off3 **lo, int *nl) {
  switch (se) {
    case SE_SEGX1D: *up = U_SEGX1D; *lo = L_SEGX1D; *nu = *nl = 1; return 0;
    case SE_SQUARE2D: *up = U_SQUARE2D; *lo = L_SQUARE2D; *nu = *nl = 4; return 0;
    case SE_CROSS2D: *up = U_CROSS2D; *lo = L_CROSS2D; *nu = *nl = 2; return 0;
    case SE_CROSS3D: *up = U_CROSS3D; *lo = L_CROSS3D; *nu = *nl = 3; return 0;
    case SE_SQUARE3D: *up = U_SQUARE3D; *lo = L_SQUARE3D; *nu = *nl = 13; return 0;
    default: return -1;
  }
}

static int dims3(int rank, const int64_t *shape, int64_t d[3]) {
  if (rank == 1) { d[0] = 1; d[1] = 1; d[2] = shape[0]; return 0; }
  if (rank == 2) { d[0] = 1; d[1] = shape[0]; d[2] = shape[1]; return 0; }
  if (rank == 3) { d[0] = shape[0]; d[1] = shape[1]; d[2] = shape[2]; return 0; }
  return -1;
}

static int elem_size(int pt) {
  switch (pt) {
    case PT_U8: return 1; case PT_U16: return 2; case PT_I32: return 4;
    case PT_F32: return 4; case PT_I64: return 8; case PT_F64: return 8;
    default: return 0;
  }
}

/* ------------------------------------------------------------------------- */
/* FIFO of linear indices (std::queue<index> in mreconstruct_t.hpp:108).       */
/* ------------------------------------------------------------------------- */
typedef struct { int64_t *buf; int64_t cap, head, tail, size; } fifo;
static int fifo_init(fifo *q, int64_t cap) {
  q->cap = cap > 16 ? cap : 16; q->head = q->tail = q->size = 0;
  q->buf = (int64_t *)malloc(sizeof(int64_t) * (size_t)q->cap);
  return q->buf ? 0 : -1;
}
static int fifo_push(fifo *q, int64_t v) {
  if (q->size == q->cap) {
    int64_t ncap = q->cap * 2;
    int64_t *nb = (int64_t *)malloc(sizeof(int64_t) * (size_t)ncap);
    if (!nb) return -1;
    for (int64_t i = 0; i < q->size; ++i) nb[i] = q->buf[(q->head + i) % q->cap];
    free(q->buf); q->buf = nb; q->head = 0; q->tail = q->size; q->cap = ncap;
  }
  q->buf[q->tail] = v; q->tail = (q->tail + 1) % q->cap; q->size++;
  return 0;
}
static int64_t fifo_pop(fifo *q) {
  int64_t v = q->buf[q->head]; q->head = (q->head + 1) % q->cap; q->size--; return v;
}

/* neighbour of linear index i (coords z,y,x) by offset o; -1 if outside (contains()) */
static inline int64_t nb_index(const int64_t d[3], int64_t z, int64_t y, int64_t x, off3 o) {
  int64_t zz = z + o.dz, yy = y + o.dy, xx = x + o.dx;
  if (zz < 0 || yy < 0 || xx < 0 || zz >= d[0] || yy >= d[1] || xx >= d[2]) return -1;
  return (zz * d[1] + yy) * d[2] + xx;
}

/* ------------------------------------------------------------------------- */
/* Type-generic bodies.                                                        */
/* ------------------------------------------------------------------------- */
#define MAXV(a, b) (((a) < (b)) ? (b) : (a)) /* std::max: returns first on ties */
#define MINV(a, b) (((b) < (a)) ? (b) : (a)) /* std::min: returns first on ties */

#define DEFINE_TYPED(T, SFX, LOWEST, HIGHEST)                                                     \
  /* generic clipped gather: t_ErodeDilateDispatcher (ero_dil_static_se_t.hpp:215-265) and      \
   * t_ErodeDilateDispatcherRuntime (ero_dil_runtime_nl_se_t.hpp:54-96).  Neighbours outside    \
   * the image are skipped (contains()), i.e. neutral padding. */                               \
  static void gather_##SFX(const int64_t d[3], const T *in, T *out, const off3 *o, int n,        \
                           int dilate) {                                                        \
    for (int64_t z = 0; z < d[0]; ++z)                                                          \
      for (int64_t y = 0; y < d[1]; ++y)                                                        \
        for (int64_t x = 0; x < d[2]; ++x) {                                                    \
          T v = dilate ? (LOWEST) : (HIGHEST);                                                  \
          for (int k = 0; k < n; ++k) {                                                         \
            int64_t j = nb_index(d, z, y, x, o[k]);                                             \
            if (j < 0) continue;                                                                \
            v = dilate ? MAXV(v, in[j]) : MINV(v, in[j]);                                       \
          }                                                                                     \
          out[(z * d[1] + y) * d[2] + x] = v;                                                   \
        }                                                                                       \
  }                                                                                             \
  /* van_herck_1d, ero_dil_line_se_t.hpp:50-89: blocks of 2k+1 starting at -k, forward and     \
   * backward partial sums (running max/min), combine f[i] = op(h[i-k], g[i+k]).                \
   * The line is padded with the neutral value (:175-187). */                                   \
  static void vhgw_line_##SFX(const T *src, T *dst, int64_t len, int64_t k, int dilate, T *f,   \
                              T *g, T *h) {                                                     \
    const int64_t alpha = 2 * k + 1, size = len + 2 * k;                                        \
    T neutral = dilate ? (LOWEST) : (HIGHEST);                                                  \
    for (int64_t i = 0; i < size; ++i) f[i] = neutral;                                          \
    memcpy(f + k, src, sizeof(T) * (size_t)len);                                                \
    for (int64_t s = 0; s < size; s += alpha) {                                                 \
      int64_t e = s + alpha < size ? s + alpha : size;                                          \
      g[s] = f[s];                                                                              \
      for (int64_t i = s + 1; i < e; ++i) g[i] = dilate ? MAXV(g[i - 1], f[i]) : MINV(g[i - 1], f[i]); \
      h[e - 1] = f[e - 1];                                                                      \
      for (int64_t i = e - 2; i >= s; --i) h[i] = dilate ? MAXV(h[i + 1], f[i]) : MINV(h[i + 1], f[i]); \
    }                                                                                           \
    for (int64_t i = 0; i < len; ++i) {                                                         \
      T a = h[i + k - k], b = g[i + k + k];                                                     \
      dst[i] = dilate ? MAXV(a, b) : MINV(a, b);                                                \
    }                                                                                           \
  }                                                                                             \
  /* t_ErodeDilateXOpLineDispatcher 1D/2D (ero_dil_line_se_t.hpp:104-190): row by row. */       \
  static int line_x_##SFX(const int64_t d[3], const T *in, T *out, int64_t k, int dilate) {     \
    int64_t rows = d[0] * d[1], len = d[2];                                                     \
    if (len == 0 || rows == 0) return 0;                                                        \
    if (k <= 0) { memcpy(out, in, sizeof(T) * (size_t)(rows * len)); return 0; }               \
    size_t ps = (size_t)(len + 2 * k);                                                          \
    T *f = (T *)malloc(ps * sizeof(T)), *g = (T *)malloc(ps * sizeof(T)),                       \
      *h = (T *)malloc(ps * sizeof(T));                                                         \
    if (!f || !g || !h) { free(f); free(g); free(h); return -2; }                               \
    for (int64_t r = 0; r < rows; ++r) vhgw_line_##SFX(in + r * len, out + r * len, len, k, dilate, f, g, h); \
    free(f); free(g); free(h);                                                                  \
    return 0;                                                                                   \
  }                                                                                             \
  /* t_transpose (pixel_processing/details/transpose_op_t.hpp:45-64) */                         \
  static void transpose_##SFX(const T *in, T *out, int64_t rows, int64_t cols) {                \
    for (int64_t y = 0; y < rows; ++y)                                                          \
      for (int64_t x = 0; x < cols; ++x) out[x * rows + y] = in[y * cols + x];                  \
  }                                                                                             \
  /* Vincent hybrid reconstruction, t_ReconstructionViewDispatcher (mreconstruct_t.hpp:84-195): \
   * clamp (select_marker), raster scan with the upper half, anti-raster scan with the lower    \
   * half + FIFO seeding, FIFO propagation.  dilate: OpRecDilate (:46-56), else OpRecErode      \
   * (:64-73). */                                                                               \
  static int recon_##SFX(const int64_t d[3], const T *marker, const T *mask, T *out, int se,    \
                         int dilate) {                                                          \
    const off3 *all, *up, *lo; int nall, nu, nl;                                                \
    nall = se_table(se, &all);                                                                  \
    if (nall < 0 || se_halves(se, &up, &nu, &lo, &nl) < 0) return -3;                           \
    const off3 *nc = all + 1; int nnc = nall - 1; /* coordinates_no_center */                   \
    int64_t N = d[0] * d[1] * d[2];                                                             \
    for (int64_t i = 0; i < N; ++i) out[i] = dilate ? MINV(marker[i], mask[i]) : MAXV(marker[i], mask[i]); \
    for (int64_t z = 0; z < d[0]; ++z)                                                          \
      for (int64_t y = 0; y < d[1]; ++y)                                                        \
        for (int64_t x = 0; x < d[2]; ++x) {                                                    \
          int64_t p = (z * d[1] + y) * d[2] + x;                                                \
          T cur = out[p];                                                                       \
          for (int k = 0; k < nu; ++k) {                                                        \
            int64_t q = nb_index(d, z, y, x, up[k]);                                            \
            if (q < 0) continue;                                                                \
            cur = dilate ? MAXV(cur, out[q]) : MINV(cur, out[q]);                               \
          }                                                                                     \
          out[p] = dilate ? MINV(cur, mask[p]) : MAXV(cur, mask[p]);                            \
        }                                                                                       \
    fifo q; if (fifo_init(&q, N / 4 + 16) < 0) return -2;                                       \
    for (int64_t z = d[0] - 1; z >= 0; --z)                                                     \
      for (int64_t y = d[1] - 1; y >= 0; --y)                                                   \
        for (int64_t x = d[2] - 1; x >= 0; --x) {                                               \
          int64_t p = (z * d[1] + y) * d[2] + x;                                                \
          T cur = out[p];                                                                       \
          for (int k = 0; k < nl; ++k) {                                                        \
            int64_t r = nb_index(d, z, y, x, lo[k]);                                            \
            if (r < 0) continue;                                                                \
            cur = dilate ? MAXV(cur, out[r]) : MINV(cur, out[r]);                               \
          }                                                                                     \
          out[p] = dilate ? MINV(cur, mask[p]) : MAXV(cur, mask[p]);                            \
          for (int k = 0; k < nl; ++k) {                                                        \
            int64_t r = nb_index(d, z, y, x, lo[k]);                                            \
            if (r < 0) continue;                                                                \
            int e1 = dilate ? (out[r] < out[p]) : (out[r] > out[p]);                            \
            int e2 = dilate ? (out[r] < mask[r]) : (out[r] > mask[r]);                          \
            if (e1 && e2) { if (fifo_push(&q, p) < 0) { free(q.buf); return -2; } }             \
          }                                                                                     \
        }                                                                                       \
    while (q.size > 0) {                                                                        \
      int64_t p = fifo_pop(&q);                                                                 \
      int64_t x = p % d[2], y = (p / d[2]) % d[1], z = p / (d[2] * d[1]);                       \
      for (int k = 0; k < nnc; ++k) {                                                           \
        int64_t r = nb_index(d, z, y, x, nc[k]);                                                \
        if (r < 0) continue;                                                                    \
        int e1 = dilate ? (out[r] < out[p]) : (out[r] > out[p]);                                \
        if (mask[r] != out[r] && e1) {                                                          \
          out[r] = dilate ? MINV(out[p], mask[r]) : MAXV(out[p], mask[r]);                      \
          if (fifo_push(&q, r) < 0) { free(q.buf); return -2; }                                 \
        }                                                                                       \
      }                                                                                         \
    }                                                                                           \
    free(q.buf);                                                                                \
    return 0;                                                                                   \
  }                                                                                             \
  /* t_low_levelingHelper (leveling_t.hpp:45-117) when low != 0, t_high_levelingHelper          \
   * (:130-202) otherwise.  The reference propagates with a priority queue keyed on the pixel   \
   * index (pq.hpp:87-93); the fixpoint does not depend on the pop order, so a FIFO is used. */ \
  static int level_##SFX(const int64_t d[3], const T *ref, const T *marker, T *out, int se,     \
                         int low) {                                                             \
    const off3 *all; int nall = se_table(se, &all);                                             \
    if (nall < 0) return -3;                                                                    \
    const off3 *nc = all + 1; int nnc = nall - 1;                                               \
    int64_t N = d[0] * d[1] * d[2];                                                             \
    memcpy(out, marker, sizeof(T) * (size_t)N);                                                 \
    fifo q; if (fifo_init(&q, N / 4 + 16) < 0) return -2;                                       \
    for (int64_t z = 0; z < d[0]; ++z)                                                          \
      for (int64_t y = 0; y < d[1]; ++y)                                                        \
        for (int64_t x = 0; x < d[2]; ++x) {                                                    \
          int64_t p = (z * d[1] + y) * d[2] + x;                                                \
          if (low ? (out[p] < ref[p]) : (out[p] > ref[p])) {                                    \
            T cur = out[p];                                                                     \
            for (int k = 0; k < nnc; ++k) {                                                     \
              int64_t r = nb_index(d, z, y, x, nc[k]);                                          \
              if (r < 0) continue;                                                              \
              cur = low ? MAXV(cur, out[r]) : MINV(cur, out[r]);                                \
            }                                                                                   \
            if (cur != out[p]) {                                                                \
              out[p] = low ? MINV(ref[p], cur) : MAXV(ref[p], cur);                             \
              if (fifo_push(&q, p) < 0) { free(q.buf); return -2; }                             \
            }                                                                                   \
          }                                                                                     \
        }                                                                                       \
    while (q.size > 0) {                                                                        \
      int64_t p = fifo_pop(&q);                                                                 \
      int64_t x = p % d[2], y = (p / d[2]) % d[1], z = p / (d[2] * d[1]);                       \
      for (int k = 0; k < nnc; ++k) {                                                           \
        int64_t r = nb_index(d, z, y, x, nc[k]);                                                \
        if (r < 0) continue;                                                                    \
        int c = low ? (out[r] < out[p] && out[r] < ref[r]) : (out[r] > out[p] && out[r] > ref[r]); \
        if (c) {                                                                                \
          T nv = low ? MINV(ref[r], out[p]) : MAXV(ref[r], out[p]);                             \
          if (out[r] != nv) {                                                                   \
            out[r] = nv;                                                                        \
            if (fifo_push(&q, r) < 0) { free(q.buf); return -2; }                               \
          }                                                                                     \
        }                                                                                       \
      }                                                                                         \
    }                                                                                           \
    free(q.buf);                                                                                \
    for (int64_t i = 0; i < N; ++i) out[i] = low ? MINV(out[i], ref[i]) : MAXV(out[i], ref[i]); \
    return 0;                                                                                   \
  }

DEFINE_TYPED(uint8_t, u8, 0, UINT8_MAX)
DEFINE_TYPED(uint16_t, u16, 0, UINT16_MAX)
DEFINE_TYPED(int32_t, i32, INT32_MIN, INT32_MAX)
DEFINE_TYPED(int64_t, i64, INT64_MIN, INT64_MAX)
DEFINE_TYPED(float, f32, -FLT_MAX, FLT_MAX)
DEFINE_TYPED(double, f64, -DBL_MAX, DBL_MAX)

#define DISPATCH(pt, CALL)                   \
  switch (pt) {                              \
    case PT_U8: CALL(uint8_t, u8); break;    \
    case PT_U16: CALL(uint16_t, u16); break; \
    case PT_I32: CALL(int32_t, i32); break;  \
    case PT_I64: CALL(int64_t, i64); break;  \
    case PT_F32: CALL(float, f32); break;    \
    case PT_F64: CALL(double, f64); break;   \
    default: return -4;                      \
  }

/* ------------------------------------------------------------------------- */
/* Public entry points (ctypes).                                               */
/* ------------------------------------------------------------------------- */

/* Erode/Dilate by an explicit offset list: poutre::Erode/Dilate(IInterface,
 * IStructuringElement, IInterface), src/low_level_morpho/ero_dil.cpp:59,152.
 * offs: n triples (dz,dy,dx). */
int or_erode_dilate_nl(int pt, int rank, const int64_t *shape, const void *in, void *out,
                       const int32_t *offs, int n, int dilate) {
  int64_t d[3];
  if (dims3(rank, shape, d) < 0) return -1;
  off3 *o = (off3 *)malloc(sizeof(off3) * (size_t)(n > 0 ? n : 1));
  if (!o) return -2;
  for (int k = 0; k < n; ++k) o[k] = (off3){offs[3 * k], offs[3 * k + 1], offs[3 * k + 2]};
  int rc = 0;
#define CALL_G(T, S) gather_##S(d, (const T *)in, (T *)out, o, n, dilate)
  switch (pt) {
    case PT_U8: CALL_G(uint8_t, u8); break;
    case PT_U16: CALL_G(uint16_t, u16); break;
    case PT_I32: CALL_G(int32_t, i32); break;
    case PT_I64: CALL_G(int64_t, i64); break;
    case PT_F32: CALL_G(float, f32); break;
    case PT_F64: CALL_G(double, f64); break;
    default: rc = -4;
  }
  free(o);
  return rc;
}

/* One static-SE pass, t_Dilate/t_Erode view switch (ero_dil_static_se_t.hpp:922-1126):
 * the window of the SE's offsets, clipped at the image border.
 *
 * SESquare3D / SECross3D: the reference routes these through slice-wise
 * specialisations (:761-915) that (1) read the buffer as ibd[2] slices of ibd[0] x ibd[1]
 * pixels and (2) keep raw pointers ptmp1..3/ptmpL to slice buffers whose storage is then
 * exchanged by imtmp.swap(...) and copy-assignments (:801-834), so from the second slice
 * on they write unrelated slices (on random data even a 3x3x3 volume differs; their own
 * test uses identical slices).  This restatement follows the SE's definition instead,
 * which is also what the reference's neighbour-list path computes with the predefined
 * se::SESquare3D / se::SECross3D (ero_dil_runtime_nl_se_t.hpp:54-96). */
static int static_pass(int pt, int rank, const int64_t *shape, const void *in, void *out, int se,
                       int dilate) {
  const off3 *tab; int n = se_table(se, &tab);
  if (n < 0 || se_rank(se) != rank) return -3;
  int64_t d[3];
  if (dims3(rank, shape, d) < 0) return -1;
#define CALL_S(T, S) gather_##S(d, (const T *)in, (T *)out, tab, n, dilate)
  DISPATCH(pt, CALL_S)
  return 0;
}

/* poutre::Erode/Dilate(IInterface, Common_NL_SE, iter, IInterface),
 * src/low_level_morpho/ero_dil_static.cpp:229-306: iter==0 copies, iter==1 one pass,
 * otherwise ping-pong through a temporary. */
int or_erode_dilate_static(int pt, int rank, const int64_t *shape, const void *in, void *out,
                           int se, int iter, int dilate) {
  int64_t d[3];
  if (iter < 0) return -1;
  if (dims3(rank, shape, d) < 0) return -1;
  int es = elem_size(pt);
  if (!es) return -4;
  size_t bytes = (size_t)(d[0] * d[1] * d[2]) * (size_t)es;
  if (iter == 0) { memcpy(out, in, bytes); return 0; }
  if (iter == 1) return static_pass(pt, rank, shape, in, out, se, dilate);
  void *tmp = malloc(bytes ? bytes : 1);
  if (!tmp) return -2;
  memcpy(tmp, in, bytes);
  int rc = 0;
  const int oddsize = iter - (iter % 2);
  for (int i = 0; i < oddsize && rc == 0; i += 2) {
    rc = static_pass(pt, rank, shape, tmp, out, se, dilate);
    if (!rc) rc = static_pass(pt, rank, shape, out, tmp, se, dilate);
  }
  if (!rc) {
    if (iter % 2 == 0) memcpy(out, tmp, bytes);
    else rc = static_pass(pt, rank, shape, tmp, out, se, dilate);
  }
  free(tmp);
  return rc;
}

/* poutre::ErodeX/DilateX/ErodeY/DilateY, src/low_level_morpho/ero_dil_line.cpp:80,144,189,252.
 * axis 0 = X (rows), axis 1 = Y (transpose -> X -> transpose, t_DilateY
 * ero_dil_line_se_t.hpp:249-282).  Y keeps the reference's restriction: its temporaries
 * have the input's shape, so t_transpose rejects non-square images
 * (transpose_op_t.hpp:59). */
int or_line(int pt, int rank, const int64_t *shape, const void *in, void *out, int64_t half,
            int axis, int dilate) {
  int64_t d[3];
  if (dims3(rank, shape, d) < 0 || rank > 2) return -1;
  if (axis == 0) {
    int rc = 0;
#define CALL_LX(T, S) rc = line_x_##S(d, (const T *)in, (T *)out, half, dilate)
    DISPATCH(pt, CALL_LX)
    return rc;
  }
  if (rank != 2) return -1;
  if (d[1] != d[2]) return -5; /* non-square: the reference throws */
  int es = elem_size(pt);
  size_t bytes = (size_t)(d[1] * d[2]) * (size_t)es;
  void *t1 = malloc(bytes ? bytes : 1), *t2 = malloc(bytes ? bytes : 1);
  if (!t1 || !t2) { free(t1); free(t2); return -2; }
  int rc = 0;
#define CALL_LY(T, S)                                                   \
  transpose_##S((const T *)in, (T *)t1, d[1], d[2]);                    \
  { int64_t dt[3] = {1, d[2], d[1]};                                    \
    rc = line_x_##S(dt, (const T *)t1, (T *)t2, half, dilate); }        \
  transpose_##S((const T *)t2, (T *)out, d[2], d[1]);
  switch (pt) {
    case PT_U8: CALL_LY(uint8_t, u8); break;
    case PT_U16: CALL_LY(uint16_t, u16); break;
    case PT_I32: CALL_LY(int32_t, i32); break;
    case PT_I64: CALL_LY(int64_t, i64); break;
    case PT_F32: CALL_LY(float, f32); break;
    case PT_F64: CALL_LY(double, f64); break;
    default: rc = -4;
  }
  free(t1); free(t2);
  return rc;
}

/* poutre::geo::Reconstruction, src/geodesy/mreconstruct.cpp:48-133 -> t_Reconstruct
 * (mreconstruct_t.hpp:493-512).  dilate != 0: reconstruction_type::dilate. */
int or_reconstruct(int pt, int rank, const int64_t *shape, const void *marker, const void *mask,
                   void *out, int se, int dilate) {
  int64_t d[3];
  if (dims3(rank, shape, d) < 0) return -1;
  if (se_rank(se) != rank) return -3;
  int rc = 0;
#define CALL_R(T, S) rc = recon_##S(d, (const T *)marker, (const T *)mask, (T *)out, se, dilate)
  DISPATCH(pt, CALL_R)
  return rc;
}

/* poutre::geo::low_leveling / high_leveling, src/geodesy/leveling.cpp:67,149. */
int or_leveling_half(int pt, int rank, const int64_t *shape, const void *ref, const void *marker,
                     void *out, int se, int low) {
  int64_t d[3];
  if (dims3(rank, shape, d) < 0) return -1;
  if (se_rank(se) != rank) return -3;
  int rc = 0;
#define CALL_L(T, S) rc = level_##S(d, (const T *)ref, (const T *)marker, (T *)out, se, low)
  DISPATCH(pt, CALL_L)
  return rc;
}

/* ------------------------------------------------------------------------- */
/* Connected-component labelling: poutre::label::label_binary / label_flat_zones */
/* (include/poutre/label/details/label_t.hpp:132-247; disjoint_min_sets :87-130). */
/* A raster scan gives each accepted pixel the provisional label of its related */
/* upper-half neighbours (merging their sets: the smaller root wins) or a new   */
/* one; roots are then numbered 1.. in creation order (min_label) and every     */
/* accepted pixel takes its root's number.  mode 0: binary (accept v != 0, or   */
/* |v| > 1e-10 for floats; a neighbour is related when it is > 0); mode 1: flat */
/* zones (every pixel accepted; related when equal).  Returns the label count.  */
/* A float neighbour in (0, 1e-10] is related but unlabelled: the reference    */
/* then reads label 0 of a possibly empty set (undefined); -5 is returned.      */
/* ------------------------------------------------------------------------- */
static int64_t dms_find(int64_t *parents, int64_t v) {
  int64_t p = parents[v];
  if (parents[p] != p) parents[v] = p = dms_find(parents, p);
  return p;
}
static int64_t dms_union(int64_t *parents, int64_t a, int64_t b) {
  const int64_t ra = dms_find(parents, a), rb = dms_find(parents, b);
  if (ra < rb) { parents[rb] = ra; return ra; }
  if (rb < ra) { parents[ra] = rb; return rb; }
  return ra;
}

#define DEFINE_LABEL(T, SFX, IS_FLOAT)                                                               \
  static int label_##SFX(const int64_t d[3], const T *in, int64_t *out, const off3 *up, int nu, int mode, \
                         int64_t *count) {                                                           \
    const int64_t n = d[0] * d[1] * d[2];                                                            \
    int64_t *parents = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));                 \
    if (!parents) return -2;                                                                         \
    int64_t np = 0;                                                                                  \
    const int64_t sentinel = INT64_MAX;                                                              \
    for (int64_t i = 0; i < n; ++i) out[i] = 0;                                                      \
    int64_t i = 0;                                                                                   \
    for (int64_t z = 0; z < d[0]; ++z)                                                               \
      for (int64_t y = 0; y < d[1]; ++y)                                                             \
        for (int64_t x = 0; x < d[2]; ++x, ++i) {                                                    \
          const T v = in[i];                                                                         \
          const int acc = mode == 1 ? 1 : (IS_FLOAT ? (fabs((double)v) > (double)ACC_EPS_##SFX) : (v != (T)0)); \
          if (!acc) continue;                                                                        \
          int64_t label = sentinel;                                                                  \
          for (int k = 0; k < nu; ++k) {                                                             \
            const int64_t j = nb_index(d, z, y, x, up[k]);                                           \
            if (j < 0) continue;                                                                     \
            const int rel = mode == 1 ? (v == in[j]) : (in[j] > (T)0);                               \
            if (!rel) continue;                                                                      \
            const int64_t nl = out[j];                                                               \
            if (nl >= np) { free(parents); return -5; }                                              \
            if (label == sentinel || label == nl) label = nl;                                        \
            else label = dms_union(parents, label, nl);                                              \
          }                                                                                          \
          if (label == sentinel) { parents[np] = np; label = np++; }                                 \
          out[i] = label;                                                                            \
        }                                                                                            \
    int64_t *num = (int64_t *)malloc(sizeof(int64_t) * (size_t)(np > 0 ? np : 1));                   \
    if (!num) { free(parents); return -2; }                                                          \
    int64_t c = 0;                                                                                   \
    for (int64_t k = 0; k < np; ++k) { if (parents[k] == k) c += 1; num[k] = c; }                    \
    for (int64_t k = 0; k < n; ++k) {                                                                \
      const T v = in[k];                                                                             \
      const int acc = mode == 1 ? 1 : (IS_FLOAT ? (fabs((double)v) > (double)ACC_EPS_##SFX) : (v != (T)0)); \
      if (acc) out[k] = num[dms_find(parents, out[k])];                                              \
    }                                                                                                \
    *count = c;                                                                                      \
    free(num);                                                                                       \
    free(parents);                                                                                   \
    return 0;                                                                                        \
  }
/* not_background<pFLOAT / pDOUBLE> thresholds (label_t.hpp:47-55) */
#define ACC_EPS_u8 0
#define ACC_EPS_u16 0
#define ACC_EPS_i32 0
#define ACC_EPS_i64 0
#define ACC_EPS_f32 1E-10F
#define ACC_EPS_f64 1E-10
DEFINE_LABEL(uint8_t, u8, 0)
DEFINE_LABEL(uint16_t, u16, 0)
DEFINE_LABEL(int32_t, i32, 0)
DEFINE_LABEL(int64_t, i64, 0)
DEFINE_LABEL(float, f32, 1)
DEFINE_LABEL(double, f64, 1)

/* upper raster half of the SE used by the labelling (split_coordinates_upper_lower of
 * neighbor_list_static_se_t.hpp; the segments' are their one earlier neighbour) */
static const off3 U_SEGX[] = {{0, 0, -1}};
static const off3 U_SEGY[] = {{0, -1, 0}};
static const off3 U_SEGZ[] = {{-1, 0, 0}};
static int label_upper(int se, const off3 **up, int *nu) {
  switch (se) {
    case SE_SEGX1D: case SE_SEGX2D: case SE_SEGX3D: *up = U_SEGX; *nu = 1; return 0;
    case SE_SEGY2D: case SE_SEGY3D: *up = U_SEGY; *nu = 1; return 0;
    case SE_SEGZ3D: *up = U_SEGZ; *nu = 1; return 0;
    case SE_SQUARE2D: *up = U_SQUARE2D; *nu = 4; return 0;
    case SE_CROSS2D: *up = U_CROSS2D; *nu = 2; return 0;
    case SE_CROSS3D: *up = U_CROSS3D; *nu = 3; return 0;
    case SE_SQUARE3D: *up = U_SQUARE3D; *nu = 13; return 0;
    default: return -1;
  }
}

int or_label(int pt, int rank, const int64_t *shape, const void *in, int64_t *out, int se, int mode,
             int64_t *count) {
  int64_t d[3];
  if (dims3(rank, shape, d) < 0) return -1;
  if (se_rank(se) != rank) return -3;
  const off3 *up;
  int nu;
  if (label_upper(se, &up, &nu) < 0) return -3;
  int rc = 0;
#define CALL_LB(T, S) rc = label_##S(d, (const T *)in, out, up, nu, mode, count)
  DISPATCH(pt, CALL_LB)
  return rc;
}

/* ------------------------------------------------------------------------- */
/* Flat 2D morphology on float32 planes with the first-in-scan-order arg      */
/* routing used for the adjoint (no counterpart in the reference; the forward */
/* is Dilate/Erode by a (2r+1)^2 square, which for r=2 equals                 */
/* Dilate(SESquare2D, iter=2)).                                               */
/* planes: number of independent H x W images stacked contiguously.           */
/* ------------------------------------------------------------------------- */
static inline int64_t argext_window(const float *img, int64_t H, int64_t W, int64_t y, int64_t x,
                                    int ry, int rx, int dilate) {
  int64_t best = -1; float bv = 0.f;
  for (int dy = -ry; dy <= ry; ++dy) {
    int64_t yy = y + dy;
    if (yy < 0 || yy >= H) continue;
    for (int dx = -rx; dx <= rx; ++dx) {
      int64_t xx = x + dx;
      if (xx < 0 || xx >= W) continue;
      float v = img[yy * W + xx];
      if (best < 0 || (dilate ? (v > bv) : (v < bv))) { best = yy * W + xx; bv = v; }
    }
  }
  return best;
}

int or_flat2d_forward(int64_t planes, int64_t H, int64_t W, const float *in, float *out, int ry,
                      int rx, int dilate) {
  for (int64_t p = 0; p < planes; ++p) {
    const float *a = in + p * H * W; float *b = out + p * H * W;
    for (int64_t y = 0; y < H; ++y)
      for (int64_t x = 0; x < W; ++x) b[y * W + x] = a[argext_window(a, H, W, y, x, ry, rx, dilate)];
  }
  return 0;
}

/* grad_in[q] = sum of grad_out[p] over outputs p whose first-in-scan-order arg-extremum is q. */
int or_flat2d_backward(int64_t planes, int64_t H, int64_t W, const float *in, const float *gout,
                       float *gin, int ry, int rx, int dilate) {
  for (int64_t p = 0; p < planes; ++p) {
    const float *a = in + p * H * W; const float *g = gout + p * H * W; float *r = gin + p * H * W;
    for (int64_t i = 0; i < H * W; ++i) r[i] = 0.f;
    for (int64_t y = 0; y < H; ++y)
      for (int64_t x = 0; x < W; ++x) r[argext_window(a, H, W, y, x, ry, rx, dilate)] += g[y * W + x];
  }
  return 0;
}
