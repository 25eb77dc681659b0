// fos_grid.cpp -- host-side grid set-up: element connectivity -> finite-volume
// face ("pair") arrays, in the order and orientation of libfosolvers.
//
// Behaviour follows polyGrid%up (polyGrid.f90:64-136: cells first, then facets;
// volumes) and polyFvGrid getNeib/sort (polyFvGrid.f90:60-227):
//   * a pair is created by the lower-numbered cell of a shared face, or by the
//     cell of a boundary face whose facet element carries the same nodes; a
//     facet wins over a neighbouring cell (the reference searches facets first);
//   * pair = [cell, neighbour], unit normal and area from the cell's face node
//     order (getINF tables, polyGrid.f90:211-278; a3p/n3p/a4p/n4p,
//     geometry.f90:17-58), so normals point out of the first element;
//   * pairs are then ordered by max(iEP) with the reference's quicksort
//     (sort.f90:15-65: middle pivot, Hoare partition), which puts the boundary
//     pairs last.
// The face matching itself is a sort of node-set keys (O(n log n)), not the
// reference's node-to-element search, so it scales to 10^7 cells.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "fos_internal.h"

namespace {

const int kTRI = 10, kQUAD = 11, kTET = 20, kHEX = 21;

int faces_of(int s) {
  if (s == kTRI || s == kQUAD) return 1;
  if (s == kTET) return 4;
  if (s == kHEX) return 6;
  return 0;
}
// local (1-based) node ids of face i of shape s; returns the node count
int face_nodes(int s, int i, int* out) {
  static const int tet[4][3] = {{1, 3, 2}, {1, 2, 4}, {1, 4, 3}, {2, 3, 4}};
  static const int hex[6][4] = {{2, 3, 7, 6}, {1, 5, 8, 4}, {3, 4, 8, 7},
                                {1, 2, 6, 5}, {5, 6, 7, 8}, {1, 4, 3, 2}};
  if (s == kTRI && i == 0) { out[0] = 1; out[1] = 2; out[2] = 3; return 3; }
  if (s == kQUAD && i == 0) { for (int k = 0; k < 4; k++) out[k] = k + 1; return 4; }
  if (s == kTET && i < 4) { for (int k = 0; k < 3; k++) out[k] = tet[i][k]; return 3; }
  if (s == kHEX && i < 6) { for (int k = 0; k < 4; k++) out[k] = hex[i][k]; return 4; }
  return 0;
}

struct Key {
  int n[4];
  bool operator<(const Key& o) const {
    for (int k = 0; k < 4; k++)
      if (n[k] != o.n[k]) return n[k] < o.n[k];
    return false;
  }
  bool operator==(const Key& o) const {
    return n[0] == o.n[0] && n[1] == o.n[1] && n[2] == o.n[2] && n[3] == o.n[3];
  }
};
Key make_key(const int* nodes, int cnt) {
  Key k;
  for (int i = 0; i < 4; i++) k.n[i] = i < cnt ? nodes[i] : 0;
  std::sort(k.n, k.n + cnt);
  return k;
}

struct Rec {
  Key key;
  int elem;  // 0-based sorted element id
  int face;  // local face
  bool operator<(const Rec& o) const {
    if (!(key == o.key)) return key < o.key;
    if (elem != o.elem) return elem < o.elem;
    return face < o.face;
  }
};

inline void sub3(const double* a, const double* b, double* o) {
  o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2];
}
inline void cross3(const double* a, const double* b, double* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
inline double len3(const double* a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

// triangle area: |(p2-p1) x (p3-p1)| / 2 ; unit normal: (p2-p1) x (p3-p2) normalised
double tri_area(const double* p1, const double* p2, const double* p3) {
  double a[3], b[3], c[3];
  sub3(p2, p1, a); sub3(p3, p1, b); cross3(a, b, c);
  return len3(c) / 2.0;
}
void tri_normal(const double* p1, const double* p2, const double* p3, double* n) {
  double a[3], b[3], c[3];
  sub3(p2, p1, a); sub3(p3, p2, b); cross3(a, b, c);
  double l = len3(c);
  n[0] = c[0] / l; n[1] = c[1] / l; n[2] = c[2] / l;
}
double tet_volume(const double* p1, const double* p2, const double* p3, const double* p4) {
  double a[3], b[3], c[3], x[3];
  sub3(p2, p1, a); sub3(p3, p1, b); sub3(p4, p1, c); cross3(b, c, x);
  return std::fabs(a[0] * x[0] + a[1] * x[1] + a[2] * x[2]) / 6.0;
}

// The reference's integer quicksort carrying a permutation (same pivot choice and
// partition steps, so equal keys end up in the same order), with an explicit stack.
void quicksort_perm(std::vector<int>& a, std::vector<int>& perm) {
  const int n = (int)a.size();
  perm.resize(n);
  for (int i = 0; i < n; i++) perm[i] = i;
  if (n < 2) return;
  std::vector<std::pair<int, int>> stack;
  stack.push_back({1, n});
  while (!stack.empty()) {
    auto [first, last] = stack.back();
    stack.pop_back();
    const int pivot = a[(first + last) / 2 - 1];
    int i = first, j = last;
    for (;;) {
      while (a[i - 1] < pivot) i++;
      while (pivot < a[j - 1]) j--;
      if (i >= j) break;
      std::swap(a[i - 1], a[j - 1]);
      std::swap(perm[i - 1], perm[j - 1]);
      i++;
      j--;
    }
    // the reference recurses into [first, i-1] before [j+1, last]; sub-ranges are
    // disjoint, so the processing order does not change the result
    if (j + 1 < last) stack.push_back({j + 1, last});
    if (first < i - 1) stack.push_back({first, i - 1});
  }
}

}  // namespace

struct fos_grid {
  int nN = 0, nE = 0, m = 0, nC = 0, nF = 0, nP = 0, nPi = 0, nPb = 0, maxFace = 0;
  std::vector<int> sE, nNE, iNE, gid, iEP, neib;
  std::vector<double> pN, p, v, aP, normP, pP;
};

extern "C" int fos_grid_build(fos_grid** out, int nN, const double* pN, int nE, int m,
                              const int* sE_in, const int* nNE_in, const int* iNE_in,
                              const int* gid_in) {
  if (!out || nN <= 0 || nE <= 0 || m <= 0 || !pN || !sE_in || !nNE_in || !iNE_in) {
    fos_set_error("fos_grid_build: bad arguments");
    return -1;
  }
  try {
    fos_grid* g = new fos_grid();
    g->nN = nN; g->nE = nE; g->m = m;
    g->pN.assign(pN, pN + 3 * (size_t)nN);
    // element order: cells, facets, others (stable)
    std::vector<int> order;
    order.reserve(nE);
    auto is_cell = [](int s) { return s == kTET || s == kHEX; };
    auto is_facet = [](int s) { return s == kTRI || s == kQUAD; };
    for (int i = 0; i < nE; i++) if (is_cell(sE_in[i])) order.push_back(i);
    g->nC = (int)order.size();
    for (int i = 0; i < nE; i++) if (is_facet(sE_in[i])) order.push_back(i);
    g->nF = (int)order.size() - g->nC;
    for (int i = 0; i < nE; i++) if (!is_cell(sE_in[i]) && !is_facet(sE_in[i])) order.push_back(i);
    g->sE.resize(nE); g->nNE.resize(nE); g->iNE.resize((size_t)m * nE); g->gid.resize(nE);
    g->p.resize(3 * (size_t)nE);
    for (int k = 0; k < nE; k++) {
      int i = order[k];
      g->sE[k] = sE_in[i];
      g->nNE[k] = nNE_in[i];
      for (int q = 0; q < m; q++) {
        int nd = iNE_in[(size_t)m * i + q];
        if (q < nNE_in[i] && (nd < 1 || nd > nN)) {
          delete g;
          fos_set_error("fos_grid_build: node id out of range");
          return -1;
        }
        g->iNE[(size_t)m * k + q] = nd;
      }
      g->gid[k] = gid_in ? gid_in[i] : 0;
      for (int d = 0; d < 3; d++) {
        double s = 0.0;
        for (int q = 0; q < nNE_in[i]; q++) s += pN[3 * (iNE_in[(size_t)m * i + q] - 1) + d];
        g->p[3 * (size_t)k + d] = s / (double)nNE_in[i];
      }
    }
    const int nC = g->nC;
    auto node = [&](int e, int local) -> const double* {
      return &g->pN[3 * (size_t)(g->iNE[(size_t)m * e + local - 1] - 1)];
    };
    // volumes
    g->v.resize(nC);
    for (int c = 0; c < nC; c++) {
      if (g->sE[c] == kTET) {
        g->v[c] = tet_volume(node(c, 1), node(c, 2), node(c, 3), node(c, 4));
      } else {  // hexahedron as six tetrahedra around the 4-6 diagonal
        static const int t[6][4] = {{1, 2, 3, 6}, {1, 3, 4, 6}, {1, 4, 5, 6},
                                    {4, 5, 6, 7}, {3, 4, 6, 7}, {4, 5, 7, 8}};
        double s = 0.0;
        for (int k = 0; k < 6; k++)
          s += tet_volume(node(c, t[k][0]), node(c, t[k][1]), node(c, t[k][2]), node(c, t[k][3]));
        g->v[c] = s;
      }
    }
    // face records
    int maxFace = 0;
    for (int e = 0; e < nE; e++) maxFace = std::max(maxFace, faces_of(g->sE[e]));
    g->maxFace = maxFace;
    std::vector<Rec> cellf, facetf;
    cellf.reserve((size_t)nC * 4);
    for (int e = 0; e < nE; e++) {
      int nf = faces_of(g->sE[e]);
      for (int f = 0; f < nf; f++) {
        int loc[4], glob[4];
        int cnt = face_nodes(g->sE[e], f, loc);
        for (int q = 0; q < cnt; q++) glob[q] = g->iNE[(size_t)m * e + loc[q] - 1];
        Rec r{make_key(glob, cnt), e, f};
        (e < nC ? cellf : facetf).push_back(r);
      }
    }
    std::sort(facetf.begin(), facetf.end());
    std::vector<Rec> cs = cellf;
    std::sort(cs.begin(), cs.end());
    // partner cell of every cell face (-1 none); cells sharing one key pair up
    std::vector<int> partner((size_t)nC * maxFace, -1), partner_face((size_t)nC * maxFace, -1);
    for (size_t a = 0; a < cs.size();) {
      size_t b = a + 1;
      while (b < cs.size() && cs[b].key == cs[a].key) b++;
      if (b - a >= 2) {
        // conforming meshes share a face between two cells; with more, pair the
        // lowest cell with the next one (the reference's search finds that one)
        const Rec& r0 = cs[a];
        const Rec& r1 = cs[a + 1];
        partner[(size_t)r0.elem * maxFace + r0.face] = r1.elem;
        partner_face[(size_t)r0.elem * maxFace + r0.face] = r1.face;
        partner[(size_t)r1.elem * maxFace + r1.face] = r0.elem;
        partner_face[(size_t)r1.elem * maxFace + r1.face] = r0.face;
      }
      a = b;
    }
    // creation order: cells ascending, faces ascending
    std::vector<int> iEP;
    std::vector<double> aP, normP, pP;
    iEP.reserve((size_t)nC * 5); aP.reserve((size_t)nC * 5 / 2);
    g->neib.assign((size_t)maxFace * nC, 0);
    for (int c = 0; c < nC; c++) {
      int nf = faces_of(g->sE[c]);
      for (int f = 0; f < nf; f++) {
        if (g->neib[(size_t)maxFace * c + f] != 0) continue;
        int loc[4], glob[4];
        int cnt = face_nodes(g->sE[c], f, loc);
        for (int q = 0; q < cnt; q++) glob[q] = g->iNE[(size_t)m * c + loc[q] - 1];
        Key k = make_key(glob, cnt);
        Rec probe{k, -1, -1};
        auto it = std::lower_bound(facetf.begin(), facetf.end(), probe);
        std::vector<int> partners;
        bool facet = false;
        for (; it != facetf.end() && it->key == k; ++it) { partners.push_back(it->elem); facet = true; }
        if (!facet) {
          int pc = partner[(size_t)c * maxFace + f];
          if (pc >= 0 && pc > c) partners.push_back(pc);
          else if (pc >= 0 && pc < c) continue;  // created by the lower cell already
        }
        for (int pe : partners) {
          g->neib[(size_t)maxFace * c + f] = pe + 1;
          if (!facet) g->neib[(size_t)maxFace * pe + partner_face[(size_t)c * maxFace + f]] = c + 1;
          iEP.push_back(c + 1);
          iEP.push_back(pe + 1);
          const double* P[4];
          for (int q = 0; q < cnt; q++) P[q] = &g->pN[3 * (size_t)(glob[q] - 1)];
          double nrm[3], ar, ctr[3];
          if (cnt == 3) {
            ar = tri_area(P[0], P[1], P[2]);
            tri_normal(P[0], P[1], P[2], nrm);
            for (int d = 0; d < 3; d++) ctr[d] = (P[0][d] + P[1][d] + P[2][d]) / 3.0;
          } else {  // quadrilateral as triangles [1,2,3] and [3,4,1]
            double n1[3], n2[3];
            ar = tri_area(P[0], P[1], P[2]) + tri_area(P[2], P[3], P[0]);
            tri_normal(P[0], P[1], P[2], n1);
            tri_normal(P[2], P[3], P[0], n2);
            for (int d = 0; d < 3; d++) nrm[d] = n1[d] + n2[d];
            double l = len3(nrm);
            for (int d = 0; d < 3; d++) nrm[d] /= l;
            for (int d = 0; d < 3; d++) ctr[d] = (P[0][d] + P[1][d] + P[2][d] + P[3][d]) / 4.0;
          }
          aP.push_back(ar);
          for (int d = 0; d < 3; d++) normP.push_back(nrm[d]);
          for (int d = 0; d < 3; d++) pP.push_back(ctr[d]);
          if (facet) g->nPb++; else g->nPi++;
        }
      }
    }
    g->nP = (int)aP.size();
    std::vector<int> key(g->nP), perm;
    for (int i = 0; i < g->nP; i++) key[i] = std::max(iEP[2 * i], iEP[2 * i + 1]);
    quicksort_perm(key, perm);
    g->iEP.resize(2 * (size_t)g->nP); g->aP.resize(g->nP);
    g->normP.resize(3 * (size_t)g->nP); g->pP.resize(3 * (size_t)g->nP);
    for (int i = 0; i < g->nP; i++) {
      int s = perm[i];
      g->iEP[2 * i] = iEP[2 * s];
      g->iEP[2 * i + 1] = iEP[2 * s + 1];
      g->aP[i] = aP[s];
      for (int d = 0; d < 3; d++) {
        g->normP[3 * i + d] = normP[3 * s + d];
        g->pP[3 * i + d] = pP[3 * s + d];
      }
    }
    *out = g;
    return 0;
  } catch (const std::exception& e) {
    fos_set_error(std::string("fos_grid_build: ") + e.what());
    return -2;
  }
}

extern "C" void fos_grid_sizes(const fos_grid* g, int* out) {
  out[0] = g->nC; out[1] = g->nE; out[2] = g->nP; out[3] = g->nPi; out[4] = g->nPb;
  out[5] = g->maxFace; out[6] = g->nF;
}

extern "C" void fos_grid_copy(const fos_grid* g, int* iEP, double* aP, double* normP,
                              double* pP, double* v, int* neib, int* gid, double* p, int* sE) {
  auto cp = [](auto* dst, const auto& src) {
    if (dst && !src.empty()) std::memcpy(dst, src.data(), src.size() * sizeof(src[0]));
  };
  cp(iEP, g->iEP); cp(aP, g->aP); cp(normP, g->normP); cp(pP, g->pP); cp(v, g->v);
  cp(neib, g->neib); cp(gid, g->gid); cp(p, g->p); cp(sE, g->sE);
}

extern "C" void fos_grid_free(fos_grid* g) { delete g; }
