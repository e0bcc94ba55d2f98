/* CPU marching cubes: the test oracle and the timed CPU baseline for the
 * mesh-extraction step of i3d/meshing.py:267-313 (convert_sdf_samples_to_ply).
 *
 * TEST INFRASTRUCTURE ONLY.  The reference calls scikit-image's
 * marching_cubes (a third-party library, not in the reference tree); this
 * file restates classic marching cubes (Lorensen & Cline 1987) with the case
 * table derived in mplicits_gb300/mc_tables.py and a canonical output order,
 * which the GPU kernel must reproduce bit for bit:
 *
 *   vertices: one per crossing edge, ordered by (grid point linear index of
 *             the edge's lower endpoint, axis);
 *   faces:    cells in linear order of their minimum point, triangles in
 *             case-table order.
 *
 * Vertex coordinate along the edge axis: ((float)idx + t) * vs + origin, with
 * t = (iso - v0) / (v1 - v0); all in float32 with separate roundings (build
 * with -ffp-contract=off).  Normals: central-difference gradient (one-sided
 * at the border) interpolated with t and normalised; values: the larger of
 * the two edge-end values.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#include "../mplicits_gb300/csrc/mc_tables.h"

static inline int inside(float v, float iso) { return v < iso; }

/* A volume is NI x N x N (C order): NI = N for the cubes of
 * i3d/meshing.py, NI < N for a slab of consecutive i-planes (the CPU
 * baseline times slabs of the grid). */
static inline int64_t lin(int64_t N, int64_t i, int64_t j, int64_t k) {
  return (i * N + j) * N + k;
}

/* Number of crossing edges owned by point (i,j,k) and its bit mask. */
static inline int point_edges(const float* S, int64_t NI, int64_t N, int64_t i, int64_t j,
                              int64_t k, float iso) {
  int64_t p = lin(N, i, j, k);
  int s = inside(S[p], iso);
  int mask = 0;
  if (i + 1 < NI && inside(S[p + N * N], iso) != s) mask |= 1;
  if (j + 1 < N && inside(S[p + N], iso) != s) mask |= 2;
  if (k + 1 < N && inside(S[p + 1], iso) != s) mask |= 4;
  return mask;
}

static inline int cell_case(const float* S, int64_t N, int64_t i, int64_t j, int64_t k,
                            float iso) {
  int c = 0;
  for (int q = 0; q < 8; ++q) {
    int64_t p = lin(N, i + (q & 1), j + ((q >> 1) & 1), k + ((q >> 2) & 1));
    c |= inside(S[p], iso) << q;
  }
  return c;
}

/* Per-slab (fixed i) vertex and triangle counts. */
void mpl_oracle_mc_count(const float* S, int64_t NI, int64_t N, float iso, int64_t* slab_verts,
                         int64_t* slab_tris) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i = 0; i < NI; ++i) {
    int64_t nv = 0, nt = 0;
    for (int64_t j = 0; j < N; ++j)
      for (int64_t k = 0; k < N; ++k) {
        nv += __builtin_popcount(point_edges(S, NI, N, i, j, k, iso));
        if (i + 1 < NI && j + 1 < N && k + 1 < N)
          nt += MPL_MC_TRI_COUNT[cell_case(S, N, i, j, k, iso)];
      }
    slab_verts[i] = nv;
    slab_tris[i] = nt;
  }
}

static float grad_axis(const float* S, int64_t NI, int64_t N, const int64_t idx[3], int axis) {
  int64_t lo[3] = {idx[0], idx[1], idx[2]};
  int64_t hi[3] = {idx[0], idx[1], idx[2]};
  if (idx[axis] > 0) lo[axis] -= 1;
  if (idx[axis] + 1 < (axis == 0 ? NI : N)) hi[axis] += 1;
  float d = S[lin(N, hi[0], hi[1], hi[2])] - S[lin(N, lo[0], lo[1], lo[2])];
  return d / (float)(hi[axis] - lo[axis]);
}

/* Vertex id of the crossing edge (point p, axis) given the exclusive prefix
 * of crossing-edge counts per point. */
static inline int64_t vertex_id(const int64_t* vprefix, const uint8_t* vmask, int64_t p,
                                int axis) {
  int m = vmask[p] & ((1 << axis) - 1);
  return vprefix[p] + __builtin_popcount(m);
}

/* Emit vertices (xyz), normals, values and faces.  slab_vbase/slab_tbase are
 * exclusive prefix sums of the counts from mpl_oracle_mc_count.  Scratch:
 * vmask [N^3] bytes and vprefix [N^3] int64. */
void mpl_oracle_mc_emit(const float* S, int64_t NI, int64_t N, float iso, float vs,
                        const float* origin, const int64_t* slab_vbase,
                        const int64_t* slab_tbase, uint8_t* vmask, int64_t* vprefix,
                        float* verts, float* normals, float* values, int32_t* faces) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i = 0; i < NI; ++i) {
    int64_t v = slab_vbase[i];
    for (int64_t j = 0; j < N; ++j)
      for (int64_t k = 0; k < N; ++k) {
        int64_t p = lin(N, i, j, k);
        int m = point_edges(S, NI, N, i, j, k, iso);
        vmask[p] = (uint8_t)m;
        vprefix[p] = v;
        for (int a = 0; a < 3; ++a) {
          if (!(m & (1 << a))) continue;
          int64_t idx0[3] = {i, j, k};
          int64_t idx1[3] = {i, j, k};
          idx1[a] += 1;
          float v0 = S[p];
          float v1 = S[lin(N, idx1[0], idx1[1], idx1[2])];
          float t = (iso - v0) / (v1 - v0);
          for (int d = 0; d < 3; ++d) {
            float c = (float)idx0[d];
            if (d == a) c = c + t;
            float x = c * vs;
            verts[3 * v + d] = x + origin[d];
          }
          float n[3];
          for (int d = 0; d < 3; ++d) {
            float g0 = grad_axis(S, NI, N, idx0, d);
            float g1 = grad_axis(S, NI, N, idx1, d);
            float dg = g1 - g0;
            float tg = t * dg;
            n[d] = g0 + tg;
          }
          float l2 = n[0] * n[0];
          l2 = l2 + n[1] * n[1];
          l2 = l2 + n[2] * n[2];
          float len = sqrtf(l2);
          for (int d = 0; d < 3; ++d) normals[3 * v + d] = len > 0.0f ? n[d] / len : 0.0f;
          values[v] = v0 > v1 ? v0 : v1;
          ++v;
        }
      }
  }
  /* faces need the vertex ids of the next slab too: second pass */
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i = 0; i < NI - 1; ++i) {
    int64_t t = slab_tbase[i];
    for (int64_t j = 0; j + 1 < N; ++j)
      for (int64_t k = 0; k + 1 < N; ++k) {
        int c = cell_case(S, N, i, j, k, iso);
        int nt = MPL_MC_TRI_COUNT[c];
        for (int q = 0; q < 3 * nt; ++q) {
          int e = MPL_MC_TRI_EDGES[c][q];
          int axis = MPL_MC_EDGE[e][0];
          int64_t p = lin(N, i + MPL_MC_EDGE[e][1], j + MPL_MC_EDGE[e][2], k + MPL_MC_EDGE[e][3]);
          faces[3 * t + q] = (int32_t)vertex_id(vprefix, vmask, p, axis);
        }
        t += nt;
      }
  }
}
