/* CPU oracle of the tubular-neighbourhood deltas (calc_deltas).
 *
 * TEST INFRASTRUCTURE ONLY: the GPU library never links or calls this file.
 *
 * Restates experiment_scripts/utils.py:46-89.  Each vertex v with unit
 * normal n keeps a radius delta and a step; every iteration displaces
 * q = v + delta * n, asks the unsigned distance D from q to the triangle
 * mesh (open3d 0.19.0 RaycastingScene.compute_distance in the reference,
 * built at experiment_scripts/train_sdf_on_neighborhood.py:145-146), and
 *   |delta - D| > eps  ->  step /= 2, delta -= step
 *   otherwise          ->  delta += step
 * while max(delta) < max_delta, for at most n_iters iterations.
 *
 * open3d is not in the reference tree and not installed.  Its distance is
 * restated as the exact distance to the nearest triangle, each triangle's
 * closest point found with the Voronoi-region method of C. Ericson,
 * "Real-Time Collision Detection" (2005), section 5.1.5, in float32 with a
 * fixed operation order (fmaf where written, nothing contracted), so that a
 * device kernel written with the same operations gives the same bits.
 * Degenerate triangles give NaN and never count as nearest.  A query point
 * with a non-finite coordinate has distance NaN, so its comparison is false
 * and its delta grows, as torch's NaN comparison does in the reference.
 *
 * Two searches give the same D bit for bit: the brute-force minimum over all
 * triangles (cell <= 0), and a uniform grid visited within delta + eps plus a
 * margin (triangles farther away cannot change the comparison).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static inline float dot3(const float* u, const float* v) {
  return fmaf(u[2], v[2], fmaf(u[1], v[1], u[0] * v[0]));
}

/* squared distance from p to triangle (a, b, c) */
static float tri_dist2(const float* p, const float* a, const float* b, const float* c) {
  float ab[3], ac[3], ap[3], bp[3], cp[3], e[3];
  for (int k = 0; k < 3; ++k) {
    ab[k] = b[k] - a[k];
    ac[k] = c[k] - a[k];
    ap[k] = p[k] - a[k];
  }
  const float d1 = dot3(ab, ap), d2 = dot3(ac, ap);
  if (d1 <= 0.f && d2 <= 0.f) return dot3(ap, ap);
  for (int k = 0; k < 3; ++k) bp[k] = p[k] - b[k];
  const float d3 = dot3(ab, bp), d4 = dot3(ac, bp);
  if (d3 >= 0.f && d4 <= d3) return dot3(bp, bp);
  const float vc = fmaf(d1, d4, -(d3 * d2));
  if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
    const float v = d1 / (d1 - d3);
    for (int k = 0; k < 3; ++k) e[k] = p[k] - fmaf(v, ab[k], a[k]);
    return dot3(e, e);
  }
  for (int k = 0; k < 3; ++k) cp[k] = p[k] - c[k];
  const float d5 = dot3(ab, cp), d6 = dot3(ac, cp);
  if (d6 >= 0.f && d5 <= d6) return dot3(cp, cp);
  const float vb = fmaf(d5, d2, -(d1 * d6));
  if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
    const float w = d2 / (d2 - d6);
    for (int k = 0; k < 3; ++k) e[k] = p[k] - fmaf(w, ac[k], a[k]);
    return dot3(e, e);
  }
  const float va = fmaf(d3, d6, -(d5 * d4));
  const float e43 = d4 - d3, e56 = d5 - d6;
  if (va <= 0.f && e43 >= 0.f && e56 >= 0.f) {
    const float w = e43 / (e43 + e56);
    for (int k = 0; k < 3; ++k) e[k] = p[k] - fmaf(w, c[k] - b[k], b[k]);
    return dot3(e, e);
  }
  const float denom = 1.0f / ((va + vb) + vc);
  const float v = vb * denom, w = vc * denom;
  for (int k = 0; k < 3; ++k) e[k] = p[k] - fmaf(ac[k], w, fmaf(ab[k], v, a[k]));
  return dot3(e, e);
}

static inline const float* vtx(const float* pos, const int32_t* faces, int64_t t, int j) {
  return pos + 3 * (int64_t)faces[3 * t + j];
}

float mpl_oracle_tri_dist(const float* p, const float* a, const float* b, const float* c) {
  return sqrtf(tri_dist2(p, a, b, c));
}

static inline int finite3(const float* q) {
  return isfinite(q[0]) && isfinite(q[1]) && isfinite(q[2]);
}

static float brute_min(const float* q, const float* pos, const int32_t* faces, int64_t T) {
  float best = INFINITY;
  for (int64_t t = 0; t < T; ++t) {
    const float d = sqrtf(tri_dist2(q, vtx(pos, faces, t, 0), vtx(pos, faces, t, 1),
                                    vtx(pos, faces, t, 2)));
    if (d < best) best = d;
  }
  return best;
}

/* unsigned distance of n points to the mesh, brute force; NaN for a point
 * with a non-finite coordinate */
void mpl_oracle_compute_distance(const float* pos, const int32_t* faces, int64_t T,
                                 const float* pts, int64_t n, float* out) {
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; ++i)
    out[i] = finite3(pts + 3 * i) ? brute_min(pts + 3 * i, pos, faces, T) : NAN;
}

/* ---- uniform grid: cells of side h over the mesh bounding box; each cell
 * lists the triangles whose (slightly grown) bounding box overlaps it ---- */
typedef struct {
  float lo[3], h;
  int64_t dim[3];
  int64_t* start; /* [cells + 1] */
  int64_t* tri;
} Grid;

static int64_t cell_of(float x, float lo, float h, int64_t dim) {
  const float f = floorf((x - lo) / h);
  if (!(f >= 0.f)) return 0;
  if (f >= (float)(dim - 1)) return dim - 1;
  return (int64_t)f;
}

static int grid_build(Grid* g, const float* pos, int64_t nv, const int32_t* faces, int64_t T,
                      float h) {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = 0; i < nv; ++i)
    for (int k = 0; k < 3; ++k) {
      lo[k] = fminf(lo[k], pos[3 * i + k]);
      hi[k] = fmaxf(hi[k], pos[3 * i + k]);
    }
  g->h = h;
  for (int k = 0; k < 3; ++k) {
    g->lo[k] = lo[k] - h;
    g->dim[k] = (int64_t)((hi[k] - lo[k]) / h) + 3;
  }
  const int64_t cells = g->dim[0] * g->dim[1] * g->dim[2];
  g->start = (int64_t*)calloc((size_t)cells + 1, sizeof(int64_t));
  if (!g->start) return -1;
  int64_t(*range)[6] = malloc(sizeof(int64_t[6]) * (size_t)(T > 0 ? T : 1));
  for (int64_t t = 0; t < T; ++t) {
    for (int k = 0; k < 3; ++k) {
      float mn = INFINITY, mx = -INFINITY;
      for (int j = 0; j < 3; ++j) {
        const float x = vtx(pos, faces, t, j)[k];
        mn = fminf(mn, x);
        mx = fmaxf(mx, x);
      }
      const float m = 1e-5f * (fabsf(mn) + fabsf(mx) + h);
      range[t][k] = cell_of(mn - m, g->lo[k], h, g->dim[k]);
      range[t][3 + k] = cell_of(mx + m, g->lo[k], h, g->dim[k]);
    }
    for (int64_t z = range[t][2]; z <= range[t][5]; ++z)
      for (int64_t y = range[t][1]; y <= range[t][4]; ++y)
        for (int64_t x = range[t][0]; x <= range[t][3]; ++x)
          g->start[(z * g->dim[1] + y) * g->dim[0] + x + 1]++;
  }
  for (int64_t c = 0; c < cells; ++c) g->start[c + 1] += g->start[c];
  g->tri = (int64_t*)malloc(sizeof(int64_t) * (size_t)(g->start[cells] > 0 ? g->start[cells] : 1));
  int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)cells);
  memcpy(fill, g->start, sizeof(int64_t) * (size_t)cells);
  for (int64_t t = 0; t < T; ++t)
    for (int64_t z = range[t][2]; z <= range[t][5]; ++z)
      for (int64_t y = range[t][1]; y <= range[t][4]; ++y)
        for (int64_t x = range[t][0]; x <= range[t][3]; ++x)
          g->tri[fill[(z * g->dim[1] + y) * g->dim[0] + x]++] = t;
  free(fill);
  free(range);
  return 0;
}

/* the minimum over the triangles listed in the cells within R of q (the
 * whole grid box around q, clamped) */
static float grid_min(const Grid* g, const float* q, float R, const float* pos,
                      const int32_t* faces) {
  int64_t a[3], b[3];
  for (int k = 0; k < 3; ++k) {
    a[k] = cell_of(q[k] - R, g->lo[k], g->h, g->dim[k]);
    b[k] = cell_of(q[k] + R, g->lo[k], g->h, g->dim[k]);
  }
  float best = INFINITY;
  for (int64_t z = a[2]; z <= b[2]; ++z)
    for (int64_t y = a[1]; y <= b[1]; ++y)
      for (int64_t x = a[0]; x <= b[0]; ++x) {
        const int64_t c = (z * g->dim[1] + y) * g->dim[0] + x;
        for (int64_t i = g->start[c]; i < g->start[c + 1]; ++i) {
          const int64_t t = g->tri[i];
          const float d = sqrtf(tri_dist2(q, vtx(pos, faces, t, 0), vtx(pos, faces, t, 1),
                                          vtx(pos, faces, t, 2)));
          if (d < best) best = d;
        }
      }
  return best;
}

/* The comparison |delta - D| > eps for D the minimum over all triangles,
 * decided as (some triangle with delta - d > eps) or (no triangle with
 * d - delta <= eps): the rounded differences are monotone in d, so both
 * forms agree.  Triangles whose bounding sphere (centroid, grown radius)
 * lies beyond delta + eps plus a margin can be neither; once a triangle with
 * d - delta <= eps is found, only those nearer than delta - eps still
 * matter; the search stops at the first triangle with delta - d > eps.  The
 * same answer as the minimum, with far fewer distance evaluations. */
static int decide_fast(const Grid* g, const float* sph, const float* q, float delta, float eps,
                       const float* pos, const int32_t* faces) {
  const float m = 1e-5f * (fmaxf(fabsf(q[0]), fmaxf(fabsf(q[1]), fabsf(q[2]))) + g->h);
  const float r_touch = (delta + eps) * 1.0001f + m;
  const float r_close = fmaxf(delta - eps, 0.f) * 1.0001f + m;
  int64_t a[3], b[3];
  for (int k = 0; k < 3; ++k) {
    a[k] = cell_of(q[k] - r_touch, g->lo[k], g->h, g->dim[k]);
    b[k] = cell_of(q[k] + r_touch, g->lo[k], g->h, g->dim[k]);
  }
  int touch = 0;
  for (int64_t z = a[2]; z <= b[2]; ++z)
    for (int64_t y = a[1]; y <= b[1]; ++y)
      for (int64_t x = a[0]; x <= b[0]; ++x) {
        const int64_t c = (z * g->dim[1] + y) * g->dim[0] + x;
        for (int64_t i = g->start[c]; i < g->start[c + 1]; ++i) {
          const int64_t t = g->tri[i];
          const float* s4 = sph + 4 * t;
          const float l = ((touch ? r_close : r_touch) + s4[3]) * 1.00002f;
          const float dx = q[0] - s4[0], dy = q[1] - s4[1], dz = q[2] - s4[2];
          if (dx * dx + dy * dy + dz * dz > l * l) continue;
          const float d = sqrtf(tri_dist2(q, vtx(pos, faces, t, 0), vtx(pos, faces, t, 1),
                                          vtx(pos, faces, t, 2)));
          if (delta - d > eps) return 1;
          if (d - delta <= eps) touch = 1;
        }
      }
  return !touch;
}

static float* spheres(const float* pos, const int32_t* faces, int64_t T, float h) {
  float* s = (float*)malloc(sizeof(float) * 4 * (size_t)(T > 0 ? T : 1));
  for (int64_t t = 0; t < T; ++t) {
    const float *p0 = vtx(pos, faces, t, 0), *p1 = vtx(pos, faces, t, 1),
                *p2 = vtx(pos, faces, t, 2);
    float c[3], r2 = 0.f;
    for (int k = 0; k < 3; ++k) c[k] = (p0[k] + p1[k] + p2[k]) / 3.f;
    const float* p[3] = {p0, p1, p2};
    for (int j = 0; j < 3; ++j) {
      const float dx = p[j][0] - c[0], dy = p[j][1] - c[1], dz = p[j][2] - c[2];
      r2 = fmaxf(r2, dx * dx + dy * dy + dz * dz);
    }
    s[4 * t] = c[0], s[4 * t + 1] = c[1], s[4 * t + 2] = c[2];
    s[4 * t + 3] = sqrtf(r2) * 1.0001f + 1e-5f * (fmaxf(fabsf(c[0]), fmaxf(fabsf(c[1]), fabsf(c[2]))) + h);
  }
  return s;
}

/* ---- bounding-volume hierarchy: triangles sorted by the Morton code of
 * their centroid (10 bits per axis over the mesh box), then split at the
 * middle of each index range down to leaves of <= 4; node boxes are the
 * exact float min/max of their triangles' corners ---- */
typedef struct {
  float lo[3], hi[3];
  int32_t left, right; /* children (internal) */
  int32_t first, count; /* triangle range in order[] (leaf: count > 0) */
} BNode;

typedef struct {
  BNode* nodes;
  int32_t* order;
  int32_t n;
} Bvh;

static uint32_t spread10(uint32_t v) {
  v &= 1023u;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

static const uint32_t* g_codes; /* qsort key (the build is single-threaded) */
static int by_code(const void* a, const void* b) {
  const uint32_t x = g_codes[*(const int32_t*)a], y = g_codes[*(const int32_t*)b];
  if (x != y) return x < y ? -1 : 1;
  return *(const int32_t*)a - *(const int32_t*)b;
}

static int32_t bvh_node(Bvh* h, const float* pos, const int32_t* faces, int32_t first,
                        int32_t count) {
  const int32_t id = h->n++;
  BNode* nd = &h->nodes[id];
  if (count <= 4) {
    nd->first = first, nd->count = count, nd->left = nd->right = -1;
    for (int k = 0; k < 3; ++k) nd->lo[k] = INFINITY, nd->hi[k] = -INFINITY;
    for (int32_t i = first; i < first + count; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          const float x = vtx(pos, faces, h->order[i], j)[k];
          nd->lo[k] = fminf(nd->lo[k], x);
          nd->hi[k] = fmaxf(nd->hi[k], x);
        }
    return id;
  }
  const int32_t half = count / 2;
  const int32_t l = bvh_node(h, pos, faces, first, half);
  const int32_t r = bvh_node(h, pos, faces, first + half, count - half);
  nd = &h->nodes[id];
  nd->left = l, nd->right = r, nd->first = 0, nd->count = 0;
  for (int k = 0; k < 3; ++k) {
    nd->lo[k] = fminf(h->nodes[l].lo[k], h->nodes[r].lo[k]);
    nd->hi[k] = fmaxf(h->nodes[l].hi[k], h->nodes[r].hi[k]);
  }
  return id;
}

static int bvh_build(Bvh* h, const float* pos, int64_t nv, const int32_t* faces, int64_t T) {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = 0; i < nv; ++i)
    for (int k = 0; k < 3; ++k) {
      lo[k] = fminf(lo[k], pos[3 * i + k]);
      hi[k] = fmaxf(hi[k], pos[3 * i + k]);
    }
  uint32_t* codes = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)T);
  h->order = (int32_t*)malloc(sizeof(int32_t) * (size_t)T);
  h->nodes = (BNode*)malloc(sizeof(BNode) * (size_t)(2 * T + 1));
  h->n = 0;
  if (!codes || !h->order || !h->nodes) return -1;
  for (int64_t t = 0; t < T; ++t) {
    uint32_t c = 0;
    for (int k = 0; k < 3; ++k) {
      const float cen = (vtx(pos, faces, t, 0)[k] + vtx(pos, faces, t, 1)[k] +
                         vtx(pos, faces, t, 2)[k]) / 3.f;
      const float ext = hi[k] - lo[k];
      float u = ext > 0.f ? (cen - lo[k]) / ext : 0.f;
      if (!(u >= 0.f)) u = 0.f; /* NaN corners map to 0 */
      if (u > 1.f) u = 1.f;
      c |= spread10((uint32_t)(u * 1023.f)) << k;
    }
    codes[t] = c;
    h->order[t] = (int32_t)t;
  }
  g_codes = codes;
  qsort(h->order, (size_t)T, sizeof(int32_t), by_code);
  free(codes);
  bvh_node(h, pos, faces, 0, (int32_t)T);
  return 0;
}

static float box_d2(const float* lo, const float* hi, const float* q) {
  float s = 0.f;
  for (int k = 0; k < 3; ++k) {
    const float g = q[k] < lo[k] ? lo[k] - q[k] : (q[k] > hi[k] ? q[k] - hi[k] : 0.f);
    s += g * g;
  }
  return s;
}

/* decide_fast's close/touch decision over the hierarchy, nearer child first */
static int decide_bvh(const Bvh* h, const float* q, float delta, float eps, const float* pos,
                      const int32_t* faces) {
  const float m = 1e-5f * (fmaxf(fabsf(q[0]), fmaxf(fabsf(q[1]), fabsf(q[2]))) + delta);
  const float r_touch = (delta + eps) * 1.0001f + m;
  const float r_close = fmaxf(delta - eps, 0.f) * 1.0001f + m;
  int32_t stack[128];
  int sp = 0, touch = 0;
  stack[sp++] = 0;
  while (sp > 0) {
    const BNode* nd = &h->nodes[stack[--sp]];
    const float lim = touch ? r_close : r_touch;
    if (box_d2(nd->lo, nd->hi, q) > lim * lim) continue;
    if (nd->count > 0) {
      for (int32_t i = nd->first; i < nd->first + nd->count; ++i) {
        const int32_t t = h->order[i];
        const float d = sqrtf(tri_dist2(q, vtx(pos, faces, t, 0), vtx(pos, faces, t, 1),
                                        vtx(pos, faces, t, 2)));
        if (delta - d > eps) return 1;
        if (d - delta <= eps) touch = 1;
      }
      continue;
    }
    const float dl = box_d2(h->nodes[nd->left].lo, h->nodes[nd->left].hi, q);
    const float dr = box_d2(h->nodes[nd->right].lo, h->nodes[nd->right].hi, q);
    /* push the farther child first so the nearer one is visited next */
    /* midpoint splits keep the depth <= 31 for T < 2^30: the stack never
       holds more than depth + 2 entries */
    if (dl <= dr) {
      stack[sp++] = nd->right;
      stack[sp++] = nd->left;
    } else {
      stack[sp++] = nd->left;
      stack[sp++] = nd->right;
    }
  }
  return !touch;
}

/* Runs calc_deltas on M vertices of C >= 6 columns (xyz, normal, ...),
 * writing [M, C + 1] rows (normal normalised, delta appended) to out.
 * step0 is the first step, max_delta / n_iters as utils.py:57 computes it in
 * max_delta's own precision, rounded to float32 (the caller computes it).
 * cell <= 0: brute-force distances; cell > 0: a grid with that cell side
 * (fast == 1: decide_fast on it, else the minimum over the cells in range);
 * fast == 2: decide_bvh on a hierarchy (cell unused).
 * force_iters >= 0 runs exactly that many iterations whatever the maximum
 * (to check a subset of a larger run, whose stopping point the whole set
 * decided).  Returns the number of iterations run, or -1 on an argument
 * error. */
int mpl_oracle_calc_deltas(const float* verts, int64_t M, int C, const float* pos, int64_t nv,
                           const int32_t* faces, int64_t T, float max_delta, float step0,
                           int n_iters, float eps, float cell, int force_iters, int fast,
                           float* out) {
  if (M <= 0 || C < 6 || n_iters < 1) return -1;
  const int64_t W = C + 1;
  float* step = (float*)malloc(sizeof(float) * (size_t)M);
  for (int64_t i = 0; i < M; ++i) {
    float* o = out + i * W;
    memcpy(o, verts + i * C, sizeof(float) * (size_t)C);
    const float len = sqrtf(o[3] * o[3] + o[4] * o[4] + o[5] * o[5]);
    o[3] = o[3] / len;
    o[4] = o[4] / len;
    o[5] = o[5] / len;
    o[C] = step0;
    step[i] = step0;
  }
  Grid g;
  memset(&g, 0, sizeof g);
  if (cell > 0.f && grid_build(&g, pos, nv, faces, T, cell) != 0) {
    free(step);
    return -1;
  }
  float* sph = cell > 0.f && fast == 1 ? spheres(pos, faces, T, cell) : NULL;
  Bvh bvh;
  memset(&bvh, 0, sizeof bvh);
  if (fast == 2 && (T >= (int64_t)1 << 30 || bvh_build(&bvh, pos, nv, faces, T) != 0)) {
    free(step);
    free(bvh.nodes);
    free(bvh.order);
    return -1;
  }
  float maxd = step0;
  int it = 0;
  while (force_iters >= 0 ? it < force_iters : (it < n_iters && maxd < max_delta)) {
    float next = -INFINITY;
#pragma omp parallel for schedule(dynamic, 64) reduction(max : next)
    for (int64_t i = 0; i < M; ++i) {
      float* o = out + i * W;
      const float delta = o[C];
      float q[3];
      for (int k = 0; k < 3; ++k) q[k] = verts[i * C + k] + delta * o[3 + k];
      int shrink = 0;
      if (finite3(q) && fast == 2) {
        shrink = decide_bvh(&bvh, q, delta, eps, pos, faces);
      } else if (finite3(q) && sph) {
        shrink = decide_fast(&g, sph, q, delta, eps, pos, faces);
      } else if (finite3(q)) {
        float D;
        if (cell > 0.f) {
          const float R = (delta + eps) * 1.0001f +
                          1e-5f * (fmaxf(fabsf(q[0]), fmaxf(fabsf(q[1]), fabsf(q[2]))) + cell);
          D = grid_min(&g, q, R, pos, faces);
        } else {
          D = brute_min(q, pos, faces, T);
        }
        shrink = fabsf(delta - D) > eps;
      }
      float s = step[i];
      if (shrink) s = s * 0.5f;
      const float nd = shrink ? delta - s : delta + s;
      step[i] = s;
      o[C] = nd;
      if (nd > next) next = nd;
    }
    maxd = next;
    ++it;
  }
  free(step);
  free(sph);
  free(bvh.nodes);
  free(bvh.order);
  free(g.start);
  free(g.tri);
  return it;
}
