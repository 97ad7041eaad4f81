// agx_mesh.cpp -- native host builders of the mesh connectivity, geometry
// and device tables (C++17, OpenMP over the host cores).
//
// The arithmetic follows the numpy restatement in mesh.py / tables.py
// operation for operation (compiled with -ffp-contract=off, no fast-math), so
// the native tables are bit-identical to it: geometry of
// abstract_2d_finite_volumes/general_mesh.py:134-267, neighbours of
// neighbour_mesh.py:296-346 (the reference builds them with a hash table in
// neighbour_table.cpp; here directed edges are bucketed by their first
// vertex), and the extrapolation geometry of
// shallow_water/sw_domain_openmp.c:1445-1484, 1684-1696.
#include <omp.h>
#include <parallel/algorithm>
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <utility>
#include <vector>
#include "../../include/agx_mesh.h"

namespace {

inline int64_t next3(int i) { return (i + 1) % 3; }

}  // namespace

extern "C" agx_status agx_mesh_geometry(int64_t n_nodes, const double* nodes, int64_t N, const int64_t* tri,
                                        int32_t use_inscribed_circle, double* V, double* E, double* C,
                                        double* normals, double* lengths, double* areas, double* radii,
                                        int64_t* first_bad) {
  if (N < 0 || n_nodes < 0 || (N > 0 && (!nodes || !tri || !V || !E || !C || !normals || !lengths || !areas || !radii)))
    return AGX_E_INVALID;
  int64_t bad = -1;
  int64_t bad_index = -1;
#pragma omp parallel for schedule(static) reduction(max : bad)
  for (int64_t k = 0; k < N; k++) {
    const int64_t a = tri[3 * k], b = tri[3 * k + 1], c = tri[3 * k + 2];
    if (a < 0 || a >= n_nodes || b < 0 || b >= n_nodes || c < 0 || c >= n_nodes) {
      bad = std::max(bad, (int64_t)1);
      continue;
    }
    const double x0 = nodes[2 * a], y0 = nodes[2 * a + 1];
    const double x1 = nodes[2 * b], y1 = nodes[2 * b + 1];
    const double x2 = nodes[2 * c], y2 = nodes[2 * c + 1];
    double* v = V + 6 * k;
    v[0] = x0; v[1] = y0; v[2] = x1; v[3] = y1; v[4] = x2; v[5] = y2;
    double* e = E + 6 * k;
    e[0] = 0.5 * (x1 + x2); e[1] = 0.5 * (y1 + y2);
    e[2] = 0.5 * (x2 + x0); e[3] = 0.5 * (y2 + y0);
    e[4] = 0.5 * (x0 + x1); e[5] = 0.5 * (y0 + y1);
    const double area = -((x1 * y0 - x0 * y1) + (x2 * y1 - x1 * y2) + (x0 * y2 - x2 * y0)) / 2.0;
    areas[k] = area;
    const double xa[3] = {x1, x2, x0}, ya[3] = {y1, y2, y0};
    const double xb[3] = {x2, x0, x1}, yb[3] = {y2, y0, y1};
    for (int i = 0; i < 3; i++) {
      double xn = xb[i] - xa[i];
      double yn = yb[i] - ya[i];
      const double ln = std::sqrt(xn * xn + yn * yn);
      xn = xn / ln;
      yn = yn / ln;
      normals[6 * k + 2 * i] = yn;
      normals[6 * k + 2 * i + 1] = -xn;
      lengths[3 * k + i] = ln;
    }
    const double cx = (x0 + x1 + x2) / 3;
    const double cy = (y0 + y1 + y2) / 3;
    C[2 * k] = cx;
    C[2 * k + 1] = cy;
    if (!use_inscribed_circle) {
      const double xm0 = (x1 + x2) / 2, ym0 = (y1 + y2) / 2;
      const double xm1 = (x2 + x0) / 2, ym1 = (y2 + y0) / 2;
      const double xm2 = (x0 + x1) / 2, ym2 = (y0 + y1) / 2;
      const double d0 = std::sqrt((cx - xm0) * (cx - xm0) + (cy - ym0) * (cy - ym0));
      const double d1 = std::sqrt((cx - xm1) * (cx - xm1) + (cy - ym1) * (cy - ym1));
      const double d2 = std::sqrt((cx - xm2) * (cx - xm2) + (cy - ym2) * (cy - ym2));
      radii[k] = std::min(std::min(d0, d1), d2);
    } else {
      const double sa = std::sqrt((x0 - x1) * (x0 - x1) + (y0 - y1) * (y0 - y1));
      const double sb = std::sqrt((x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2));
      const double sc = std::sqrt((x2 - x0) * (x2 - x0) + (y2 - y0) * (y2 - y0));
      radii[k] = 2.0 * area / (sa + sb + sc);
    }
  }
  if (bad > 0) return AGX_E_INVALID;   // vertex index out of range
  for (int64_t k = 0; k < N; k++)
    if (!(areas[k] > 0.0)) { bad_index = k; break; }
  if (first_bad) *first_bad = bad_index;
  return AGX_OK;
}

extern "C" agx_status agx_mesh_neighbours(int64_t n_nodes, int64_t N, const int64_t* tri, int64_t* nb, int64_t* ne,
                                          int64_t* n_boundaries) {
  if (N < 0 || n_nodes < 0 || (N > 0 && (!tri || !nb || !ne || !n_boundaries))) return AGX_E_INVALID;
  for (int64_t s = 0; s < 3 * N; s++)
    if (tri[s] < 0 || tri[s] >= n_nodes) return AGX_E_INVALID;
  // directed edge of slot s = 3k + i runs from v[(i+1)%3] to v[(i+2)%3];
  // bucket the slots by their first vertex (CSR)
  std::vector<std::atomic<int64_t>> count(n_nodes + 1);
  for (auto& c : count) c.store(0, std::memory_order_relaxed);
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < 3 * N; s++) {
    const int64_t k = s / 3;
    const int i = (int)(s - 3 * k);
    count[tri[3 * k + next3(i)] + 1].fetch_add(1, std::memory_order_relaxed);
  }
  std::vector<int64_t> start(n_nodes + 1, 0);
  for (int64_t v = 0; v < n_nodes; v++) start[v + 1] = start[v] + count[v + 1].load(std::memory_order_relaxed);
  for (int64_t v = 0; v <= n_nodes; v++) count[v].store(start[v], std::memory_order_relaxed);
  std::vector<int64_t> bucket(3 * N);
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < 3 * N; s++) {
    const int64_t k = s / 3;
    const int i = (int)(s - 3 * k);
    const int64_t a = tri[3 * k + next3(i)];
    bucket[count[a].fetch_add(1, std::memory_order_relaxed)] = s;
  }
  auto head = [&](int64_t s) { return tri[3 * (s / 3) + next3((int)(s % 3))]; };
  auto tail = [&](int64_t s) { return tri[3 * (s / 3) + (s % 3 + 2) % 3]; };
  int dup = 0;
#pragma omp parallel for schedule(static) reduction(| : dup)
  for (int64_t v = 0; v < n_nodes; v++) {
    for (int64_t p = start[v]; p < start[v + 1]; p++)
      for (int64_t q = p + 1; q < start[v + 1]; q++)
        if (tail(bucket[p]) == tail(bucket[q])) dup = 1;
  }
  if (dup) return AGX_E_STATE;           // a directed edge appears twice
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < N; k++) {
    int64_t nbound = 0;
    for (int i = 0; i < 3; i++) {
      const int64_t s = 3 * k + i;
      const int64_t a = head(s), b = tail(s);
      int64_t hit = -1;
      for (int64_t p = start[b]; p < start[b + 1]; p++)
        if (tail(bucket[p]) == a) { hit = bucket[p]; break; }
      nb[s] = hit >= 0 ? hit / 3 : -1;
      ne[s] = hit >= 0 ? hit % 3 : -1;
      if (hit < 0) nbound++;
    }
    n_boundaries[k] = nbound;
  }
  return AGX_OK;
}

extern "C" agx_status agx_sfc_order(int64_t n, const double* pts, int32_t curve, int32_t bits, int64_t* order) {
  if (n < 0 || (n > 0 && (!pts || !order)) || bits < 1 || bits > 30 || (curve != 0 && curve != 1)) return AGX_E_INVALID;
  if (n == 0) return AGX_OK;
  double lo[2] = {pts[0], pts[1]}, hi[2] = {pts[0], pts[1]};
  for (int64_t j = 1; j < n; j++)
    for (int c = 0; c < 2; c++) {
      lo[c] = std::min(lo[c], pts[2 * j + c]);
      hi[c] = std::max(hi[c], pts[2 * j + c]);
    }
  const double span[2] = {std::max(hi[0] - lo[0], 1e-300), std::max(hi[1] - lo[1], 1e-300)};
  std::vector<std::pair<int64_t, int64_t>> key(n);
  const int64_t full = (int64_t(1) << bits) - 1;
  if (curve == 0) {
    auto spread = [](uint64_t v) {
      v &= 0xFFFFull;
      v = (v | (v << 8)) & 0x00FF00FFull;
      v = (v | (v << 4)) & 0x0F0F0F0Full;
      v = (v | (v << 2)) & 0x33333333ull;
      v = (v | (v << 1)) & 0x55555555ull;
      return v;
    };
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n; j++) {
      uint64_t q[2];
      for (int c = 0; c < 2; c++) {
        const double t = (pts[2 * j + c] - lo[c]) / span[c] * (double)full;
        uint64_t u = (uint64_t)t;
        q[c] = std::min<uint64_t>(u, (uint64_t)full);
      }
      key[j] = {(int64_t)(spread(q[0]) | (spread(q[1]) << 1)), j};
    }
  } else {
    const int64_t nn = int64_t(1) << bits;
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n; j++) {
      int64_t x = (int64_t)((pts[2 * j] - lo[0]) / span[0] * (double)(nn - 1));
      int64_t y = (int64_t)((pts[2 * j + 1] - lo[1]) / span[1] * (double)(nn - 1));
      x = std::min(std::max(x, (int64_t)0), nn - 1);
      y = std::min(std::max(y, (int64_t)0), nn - 1);
      int64_t d = 0;
      for (int64_t s = nn / 2; s > 0; s /= 2) {
        const int64_t rx = (x & s) > 0 ? 1 : 0;
        const int64_t ry = (y & s) > 0 ? 1 : 0;
        d += s * s * ((3 * rx) ^ ry);
        const bool flip = !ry;
        const int64_t sx = (flip && rx) ? s - 1 - x : x;
        const int64_t sy = (flip && rx) ? s - 1 - y : y;
        x = flip ? sy : sx;
        y = flip ? sx : sy;
      }
      key[j] = {d, j};
    }
  }
  __gnu_parallel::sort(key.begin(), key.end());     // (key, index) pairs: a stable order by key
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < n; j++) order[j] = key[j].second;
  return AGX_OK;
}

extern "C" agx_status agx_tile_halos(int64_t N, const int32_t* conn, int32_t tile, int32_t halo_max, int32_t inline_id,
                                     int32_t* lnk, int32_t* halo_off, int32_t* halo_cnt, int32_t* halo_cells,
                                     int64_t halo_capacity, int64_t* n_halo, int64_t* n_halo_unclamped) {
  if (N < 0 || tile <= 0 || halo_max < 0 || (N > 0 && (!conn || !lnk || !halo_off || !halo_cnt))) return AGX_E_INVALID;
  const int64_t T = (N + tile - 1) / tile;
  std::vector<std::vector<int32_t>> lists(T);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t t = 0; t < T; t++) {
    const int64_t k0 = t * tile, k1 = std::min(N, k0 + tile);
    std::vector<int32_t>& L = lists[t];
    for (int64_t k = k0; k < k1; k++)
      for (int i = 0; i < 3; i++) {
        const int32_t n = conn[4 * k + i];
        if (n >= 0 && n / tile != t) L.push_back(n);
      }
    std::sort(L.begin(), L.end());
    L.erase(std::unique(L.begin(), L.end()), L.end());
    for (int64_t k = k0; k < k1; k++) {
      int32_t loc[3];
      for (int i = 0; i < 3; i++) {
        const int32_t n = conn[4 * k + i];
        if (n < 0) {
          loc[i] = inline_id;
        } else if (n / tile == t) {
          loc[i] = (int32_t)(n - k0);
        } else {
          const int64_t pos = std::lower_bound(L.begin(), L.end(), n) - L.begin();
          loc[i] = pos < halo_max ? (int32_t)(tile + pos) : inline_id;
        }
      }
      lnk[k] = loc[0] | (loc[1] << 10) | (loc[2] << 20);
    }
  }
  int64_t off = 0, total = 0;
  for (int64_t t = 0; t < T; t++) {
    const int64_t c = std::min<int64_t>((int64_t)lists[t].size(), halo_max);
    halo_off[t] = (int32_t)off;
    halo_cnt[t] = (int32_t)c;
    off += c;
    total += (int64_t)lists[t].size();
  }
  if (n_halo) *n_halo = off;
  if (n_halo_unclamped) *n_halo_unclamped = total;
  if (halo_cells) {
    if (off > halo_capacity) return AGX_E_INVALID;
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < T; t++)
      for (int64_t j = 0; j < halo_cnt[t]; j++) halo_cells[halo_off[t] + j] = lists[t][j];
  }
  return AGX_OK;
}

extern "C" agx_status agx_pack_plain(int64_t N, const int64_t* nb, const int64_t* ne, const int64_t* sn,
                                     const int64_t* nbnd, const int64_t* full, const uint8_t* per_side_in,
                                     const int64_t* orig, const double* normals, const double* lengths,
                                     const double* C, const double* Em, int32_t* conn, int32_t* surr, double* geo,
                                     int32_t* edge_slot, int32_t* edge_opp, int64_t* n_edges) {
  if (N < 0 || (N > 0 && (!nb || !ne || !sn || !nbnd || !normals || !lengths || !C || !Em || !conn || !surr ||
                          !geo || !edge_slot || !edge_opp || !n_edges)))
    return AGX_E_INVALID;
  if (N >= (int64_t(1) << 29)) return AGX_E_INVALID;
  std::vector<uint8_t> ps(3 * N, 0);
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < 3 * N; s++) {
    const int64_t k = s / 3;
    const int i = (int)(s % 3);
    bool p = per_side_in ? per_side_in[s] != 0 : false;
    if (nb[s] >= 0) {
      const int64_t n = nb[s], m = ne[s];
      const bool mirror = normals[6 * k + 2 * i] == -normals[6 * n + 2 * m] &&
                          normals[6 * k + 2 * i + 1] == -normals[6 * n + 2 * m + 1] && lengths[s] == lengths[3 * n + m];
      const bool back = nb[3 * n + m] == k;
      if (!(mirror && back)) p = true;
    }
    ps[s] = p;
  }
  std::vector<uint8_t> ps2(ps);
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < 3 * N; s++)
    if (nb[s] >= 0 && ps[3 * nb[s] + ne[s]]) ps2[s] = 1;
  std::vector<int64_t> cnt(N + 1, 0);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < N; k++) {
    int64_t meta = 0, own = 0;
    for (int i = 0; i < 3; i++) {
      const int64_t s = 3 * k + i;
      const bool interior = nb[s] >= 0;
      meta |= ((interior ? ne[s] : 0) & 3) << (2 * i);
      meta |= (int64_t)ps2[s] << (9 + i);
      const int64_t sv = sn[s];
      const int64_t ok = orig ? orig[k] : k, osv = orig ? orig[sv] : sv;
      const bool before = (sv != k) && (osv < ok);
      meta |= (int64_t)before << (12 + i);
      if (!interior || ps2[s] || k < nb[s]) own++;
      conn[4 * k + i] = (int32_t)nb[s];
      surr[4 * k + i] = (int32_t)sn[s];
    }
    meta |= ((full ? full[k] : 1) & 1) << 8;
    meta |= (nbnd[k] & 3) << 16;
    conn[4 * k + 3] = (int32_t)meta;
    surr[4 * k + 3] = (int32_t)nbnd[k];
    cnt[k + 1] = own;
  }
  for (int64_t k = 0; k < N; k++) cnt[k + 1] += cnt[k];
  *n_edges = cnt[N];
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < N; k++) {
    int64_t p = cnt[k];
    for (int i = 0; i < 3; i++) {
      const int64_t s = 3 * k + i;
      const bool interior = nb[s] >= 0;
      if (!interior || ps2[s] || k < nb[s]) {
        edge_slot[p] = (int32_t)s;
        edge_opp[p] = (interior && !ps2[s]) ? (int32_t)(3 * nb[s] + ne[s]) : -1;
        p++;
      }
    }
    // extrapolation geometry
    double* g = geo + 11 * k;
    const double x = C[2 * k], y = C[2 * k + 1];
    for (int i = 0; i < 3; i++) {
      g[i] = Em[6 * k + 2 * i] - x;
      g[3 + i] = Em[6 * k + 2 * i + 1] - y;
    }
    for (int i = 6; i < 11; i++) g[i] = 0.0;
    const int64_t* s = sn + 3 * k;
    if (nbnd[k] <= 1) {
      const double x0 = C[2 * s[0]], y0 = C[2 * s[0] + 1];
      const double x1 = C[2 * s[1]], y1 = C[2 * s[1] + 1];
      const double x2 = C[2 * s[2]], y2 = C[2 * s[2] + 1];
      const double dx1 = x1 - x0, dx2 = x2 - x0, dy1 = y1 - y0, dy2 = y2 - y0;
      const double area2 = dy2 * dx1 - dy1 * dx2;
      g[6] = dx1;
      g[7] = dx2;
      g[8] = dy1;
      g[9] = dy2;
      g[10] = 1.0 / area2;
    } else if (nbnd[k] == 2) {
      const int j = s[0] != k ? 0 : (s[1] != k ? 1 : 2);
      const int64_t kn = s[j];
      const double ddx = C[2 * kn] - x, ddy = C[2 * kn + 1] - y;
      const double dist2 = ddx * ddx + ddy * ddy;
      double gdx = 1.0 / dist2;
      const double gdy = gdx * ddy;
      gdx = gdx * ddx;
      g[6] = gdx;
      g[7] = gdy;
    }
  }
  return AGX_OK;
}

extern "C" agx_status agx_pack_mixed(int64_t N, const int64_t* order, const int64_t* nb, const int64_t* ne,
                                     const int64_t* sn, const int64_t* nbnd, const double* C, const double* Em,
                                     const double* V, const double* radii, const double* areas, int32_t* conn,
                                     float* geo, double* area_s, int32_t* order_s) {
  if (N < 0 || (N > 0 && (!order || !nb || !ne || !sn || !nbnd || !C || !Em || !V || !radii || !areas || !conn ||
                          !geo || !area_s || !order_s)))
    return AGX_E_INVALID;
  std::vector<int64_t> inv(N);
  for (int64_t j = 0; j < N; j++) {
    if (order[j] < 0 || order[j] >= N) return AGX_E_INVALID;
    inv[order[j]] = j;
  }
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < N; j++) {
    const int64_t k = order[j];
    const double cx = C[2 * k], cy = C[2 * k + 1];
    double dxv[3], dyv[3];
    for (int i = 0; i < 3; i++) {
      dxv[i] = Em[6 * k + 2 * i] - cx;
      dyv[i] = Em[6 * k + 2 * i + 1] - cy;
    }
    double M[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    const int64_t* s = sn + 3 * k;
    if (nbnd[k] <= 1) {
      const double x0 = C[2 * s[0]], y0 = C[2 * s[0] + 1];
      const double x1 = C[2 * s[1]], y1 = C[2 * s[1] + 1];
      const double x2 = C[2 * s[2]], y2 = C[2 * s[2] + 1];
      const double dx1 = x1 - x0, dx2 = x2 - x0, dy1 = y1 - y0, dy2 = y2 - y0;
      const double area2 = dy2 * dx1 - dy1 * dx2;
      const double ia2 = 1.0 / area2;
      const double gx[3] = {(dy1 - dy2) * ia2, dy2 * ia2, -dy1 * ia2};
      const double gy[3] = {(dx2 - dx1) * ia2, -dx2 * ia2, dx1 * ia2};
      for (int i = 0; i < 3; i++)
        for (int c = 0; c < 3; c++) M[i][c] = gx[c] * dxv[i] + gy[c] * dyv[i];
    } else if (nbnd[k] == 2) {
      const int jj = s[0] != k ? 0 : (s[1] != k ? 1 : 2);
      const int64_t kn = s[jj];
      const double ddx = C[2 * kn] - cx, ddy = C[2 * kn + 1] - cy;
      const double dist2 = ddx * ddx + ddy * ddy;
      const double gdx = ddx / dist2, gdy = ddy / dist2;
      for (int i = 0; i < 3; i++) M[i][jj] = gdx * dxv[i] + gdy * dyv[i];
    }
    float* g = geo + 16 * j;
    for (int i = 0; i < 3; i++)
      for (int c = 0; c < 3; c++) g[3 * i + c] = (float)M[i][c];
    const double* v = V + 6 * k;
    g[9] = (float)(v[4] - v[2]);
    g[10] = (float)(v[5] - v[3]);
    g[11] = (float)(v[0] - v[4]);
    g[12] = (float)(v[1] - v[5]);
    g[13] = (float)(v[2] - v[0]);
    g[14] = (float)(v[3] - v[1]);
    g[15] = (float)radii[k];
    int64_t meta = 0;
    for (int i = 0; i < 3; i++) {
      const int64_t n = nb[3 * k + i];
      meta |= ((n >= 0 ? ne[3 * k + i] : 0) & 3) << (2 * i);
      conn[4 * j + i] = (int32_t)(n >= 0 ? inv[n] : n);
    }
    meta |= int64_t(1) << 8;
    meta |= (nbnd[k] & 3) << 16;
    conn[4 * j + 3] = (int32_t)meta;
    area_s[j] = areas[k];
    order_s[j] = (int32_t)k;
  }
  return AGX_OK;
}

extern "C" int32_t agx_mesh_threads(int32_t n) {
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
}
