// Host-side integer structure of the MGPBD system (see structure.h).
//
// The tet aggregation of the reference (cons/tet_aggregation.py:40-127)
// breaks ties by the iteration order of CPython `set` objects of small
// integers: `sorted(adj[seed] - visited, key=degree)` is a stable sort over
// the set-difference result, and `for nb2 in adj[nb]` walks a set.  For
// integers hash(i) == i, so that order is the slot order of CPython's open
// addressing table (Objects/setobject.c: 8-slot minimum table, 9 linear
// probes when they fit, then the perturbed recurrence i = 5i + 1 + perturb
// with perturb >>= 5, growth when fill*5 >= mask*3).  SetEmu below models
// exactly the operations the reference performs (add, membership,
// difference into a new set, iteration), which makes the aggregate ids
// identical to the reference's; the golden fixtures check it on grids,
// balls and the reference's own meshes.
#include "structure.h"

#include <algorithm>
#include <array>
#include <cstring>
#include <numeric>
#include <stdexcept>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace mgpbd {

namespace {

constexpr int32_t kEmpty = -1;
constexpr int32_t kDummy = -2;
constexpr size_t kLinearProbes = 9;
constexpr int kPerturbShift = 5;

// Model of a CPython set holding non-negative ints (hash(i) == i).
struct SetEmu {
  std::vector<int32_t> slot;
  size_t mask = 7;
  int64_t fill = 0;
  int64_t used = 0;

  SetEmu() : slot(8, kEmpty) {}

  static void insert_clean(std::vector<int32_t>& tab, size_t mask, int32_t key) {
    size_t perturb = static_cast<size_t>(key);
    size_t i = static_cast<size_t>(key) & mask;
    while (true) {
      size_t e = i;
      if (tab[e] == kEmpty) { tab[e] = key; return; }
      if (i + kLinearProbes <= mask) {
        for (size_t j = 0; j < kLinearProbes; ++j) {
          ++e;
          if (tab[e] == kEmpty) { tab[e] = key; return; }
        }
      }
      perturb >>= kPerturbShift;
      i = (i * 5 + 1 + perturb) & mask;
    }
  }

  void resize(int64_t minused) {
    size_t newsize = 8;
    while (newsize <= static_cast<size_t>(minused)) newsize <<= 1;
    std::vector<int32_t> old;
    old.swap(slot);
    slot.assign(newsize, kEmpty);
    mask = newsize - 1;
    if (fill != used) fill = used;
    for (int32_t k : old)
      if (k >= 0) insert_clean(slot, mask, k);
  }

  void add(int32_t key) {
    size_t perturb = static_cast<size_t>(key);
    size_t i = static_cast<size_t>(key) & mask;
    int64_t freeslot = -1;
    while (true) {
      size_t e = i;
      size_t probes = (i + kLinearProbes <= mask) ? kLinearProbes : 0;
      while (true) {
        int32_t k = slot[e];
        if (k == kEmpty) {
          if (freeslot >= 0) {
            ++used;
            slot[freeslot] = key;
            return;
          }
          ++fill;
          ++used;
          slot[e] = key;
          if (fill * 5 < static_cast<int64_t>(mask) * 3) return;
          resize(used > 50000 ? used * 2 : used * 4);
          return;
        }
        if (k == key) return;
        if (k == kDummy && freeslot < 0) freeslot = static_cast<int64_t>(e);
        if (probes == 0) break;
        --probes;
        ++e;
      }
      perturb >>= kPerturbShift;
      i = (i * 5 + 1 + perturb) & mask;
    }
  }

  bool discard(int32_t key) {
    size_t perturb = static_cast<size_t>(key);
    size_t i = static_cast<size_t>(key) & mask;
    while (true) {
      size_t e = i;
      size_t probes = (i + kLinearProbes <= mask) ? kLinearProbes : 0;
      while (true) {
        int32_t k = slot[e];
        if (k == kEmpty) return false;
        if (k == key) {
          slot[e] = kDummy;
          --used;
          return true;
        }
        if (probes == 0) break;
        --probes;
        ++e;
      }
      perturb >>= kPerturbShift;
      i = (i * 5 + 1 + perturb) & mask;
    }
  }

  // set(other) / other.copy(): make_new_set -> set_merge into an empty set.
  static SetEmu copy_of(const SetEmu& o) {
    SetEmu s;
    if (o.used == 0) return s;
    if ((s.fill + o.used) * 5 >= static_cast<int64_t>(s.mask) * 3) s.resize((s.used + o.used) * 2);
    if (s.fill == 0 && s.mask == o.mask && o.fill == o.used) {
      s.slot = o.slot;
      s.fill = o.fill;
      s.used = o.used;
      return s;
    }
    s.fill = o.used;
    s.used = o.used;
    for (int32_t k : o.slot)
      if (k >= 0) insert_clean(s.slot, s.mask, k);
    return s;
  }

  template <class F>
  void for_each(F&& f) const {
    for (int32_t k : slot)
      if (k >= 0) f(k);
  }
};

struct FaceRec {
  int32_t a, b, c;
  int32_t tet;
  int64_t occ;  // 4 * tet + dropped slot: order of first appearance
};

}  // namespace

// ---------------------------------------------------------------------------
// cons/mgpbd_gpu.py:153-194
Csr build_pattern(const int32_t* t_i, int32_t nt) {
  int32_t nv = 0;
  for (int64_t k = 0; k < 4LL * nt; ++k) {
    if (t_i[k] < 0) throw std::invalid_argument("negative vertex id in t_i");
    nv = std::max(nv, t_i[k] + 1);
  }
  // vertex -> sorted unique tets (vert_to_tets sets)
  std::vector<int32_t> vptr(nv + 1, 0), vent;
  for (int64_t k = 0; k < 4LL * nt; ++k) vptr[t_i[k] + 1]++;
  for (int32_t v = 0; v < nv; ++v) vptr[v + 1] += vptr[v];
  vent.resize(vptr[nv]);
  {
    std::vector<int32_t> cur(vptr.begin(), vptr.end() - 1);
    for (int32_t t = 0; t < nt; ++t)
      for (int l = 0; l < 4; ++l) {
        int32_t v = t_i[4LL * t + l];
        // a tet listing a vertex twice is stored once (set semantics)
        if (cur[v] > vptr[v] && vent[cur[v] - 1] == t) continue;
        vent[cur[v]++] = t;
      }
    // compact rows whose duplicates were skipped
    std::vector<int32_t> nptr(nv + 1, 0);
    for (int32_t v = 0; v < nv; ++v) nptr[v + 1] = nptr[v] + (cur[v] - vptr[v]);
    if (nptr[nv] != vptr[nv]) {
      std::vector<int32_t> nent(nptr[nv]);
      for (int32_t v = 0; v < nv; ++v)
        std::copy(vent.begin() + vptr[v], vent.begin() + cur[v], nent.begin() + nptr[v]);
      vent.swap(nent);
      vptr.swap(nptr);
    }
  }
  Csr p;
  p.n_rows = p.n_cols = nt;
  p.indptr.assign(nt + 1, 0);
  std::vector<int32_t> cnt(nt, 0);
  auto row = [&](int32_t t, std::vector<int32_t>& buf) {
    buf.clear();
    for (int l = 0; l < 4; ++l) {
      int32_t v = t_i[4LL * t + l];
      buf.insert(buf.end(), vent.begin() + vptr[v], vent.begin() + vptr[v + 1]);
    }
    std::sort(buf.begin(), buf.end());
    buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
    buf.erase(std::remove(buf.begin(), buf.end(), t), buf.end());
  };
#pragma omp parallel
  {
    std::vector<int32_t> buf;
#pragma omp for schedule(static)
    for (int32_t t = 0; t < nt; ++t) {
      row(t, buf);
      cnt[t] = static_cast<int32_t>(buf.size()) + 1;
    }
  }
  int64_t total = 0;
  for (int32_t t = 0; t < nt; ++t) {
    total += cnt[t];
    if (total > INT32_MAX) throw std::length_error("nnz exceeds int32");
    p.indptr[t + 1] = static_cast<int32_t>(total);
  }
  p.indices.resize(total);
#pragma omp parallel
  {
    std::vector<int32_t> buf;
#pragma omp for schedule(static)
    for (int32_t t = 0; t < nt; ++t) {
      row(t, buf);
      int32_t* dst = p.indices.data() + p.indptr[t];
      std::copy(buf.begin(), buf.end(), dst);
      dst[buf.size()] = t;  // diagonal last
    }
  }
  return p;
}

// ---------------------------------------------------------------------------
// cons/tet_aggregation.py:11-37: tets sharing a face that exactly two tets
// have, as (first appearance of the face, tet, tet), in order of first
// appearance (the order the reference fills its adjacency sets in).
struct FacePair {
  int64_t first;
  int32_t t0, t1;
};

static std::vector<FacePair> face_pairs(const int32_t* t_i, int32_t nt) {
  // faces keyed by the sorted vertex triple, in order of first appearance
  std::vector<FaceRec> faces(4LL * nt);
  for (int32_t t = 0; t < nt; ++t) {
    for (int skip = 0; skip < 4; ++skip) {
      std::array<int32_t, 3> f{};
      int m = 0;
      for (int j = 0; j < 4; ++j)
        if (j != skip) f[m++] = t_i[4LL * t + j];
      std::sort(f.begin(), f.end());
      faces[4LL * t + skip] = FaceRec{f[0], f[1], f[2], t, 4LL * t + skip};
    }
  }
  std::sort(faces.begin(), faces.end(), [](const FaceRec& x, const FaceRec& y) {
    if (x.a != y.a) return x.a < y.a;
    if (x.b != y.b) return x.b < y.b;
    if (x.c != y.c) return x.c < y.c;
    return x.occ < y.occ;
  });
  std::vector<FacePair> pairs;
  pairs.reserve(2LL * nt);
  for (size_t s = 0; s < faces.size();) {
    size_t e = s + 1;
    while (e < faces.size() && faces[e].a == faces[s].a && faces[e].b == faces[s].b &&
           faces[e].c == faces[s].c)
      ++e;
    if (e - s == 2) pairs.push_back({faces[s].occ, faces[s].tet, faces[s + 1].tet});
    s = e;
  }
  std::sort(pairs.begin(), pairs.end(),
            [](const FacePair& x, const FacePair& y) { return x.first < y.first; });
  return pairs;
}

Csr face_adjacency(const int32_t* t_i, int32_t nt) {
  const std::vector<FacePair> pairs = face_pairs(t_i, nt);
  Csr a;
  a.n_rows = a.n_cols = nt;
  a.indptr.assign(nt + 1, 0);
  for (const FacePair& p : pairs) {
    ++a.indptr[p.t0 + 1];
    ++a.indptr[p.t1 + 1];
  }
  for (int32_t t = 0; t < nt; ++t) a.indptr[t + 1] += a.indptr[t];
  a.indices.resize(a.indptr[nt]);
  std::vector<int32_t> fill(a.indptr.begin(), a.indptr.end() - 1);
  for (const FacePair& p : pairs) {
    a.indices[fill[p.t0]++] = p.t1;
    a.indices[fill[p.t1]++] = p.t0;
  }
  for (int32_t t = 0; t < nt; ++t)
    std::sort(a.indices.begin() + a.indptr[t], a.indices.begin() + a.indptr[t + 1]);
  return a;
}

// cons/tet_aggregation.py:40-127 (pass 1).
int32_t tet_aggregate(const int32_t* t_i, int32_t nt, int32_t max_agg_size,
                      std::vector<int32_t>& agg_ids) {
  const std::vector<FacePair> pairs = face_pairs(t_i, nt);
  std::vector<SetEmu> adj(nt);
  for (const FacePair& p : pairs) {
    adj[p.t0].add(p.t1);
    adj[p.t1].add(p.t0);
  }
  std::vector<int64_t> deg(nt);
  for (int32_t t = 0; t < nt; ++t) deg[t] = adj[t].used;

  std::vector<int32_t> order(nt);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t x, int32_t y) { return deg[x] < deg[y]; });

  agg_ids.assign(nt, -1);
  std::vector<uint8_t> visited(nt, 0);
  int64_t n_visited = 0;
  int32_t n_agg = 0;
  std::vector<int32_t> cand;
  for (int32_t seed : order) {
    if (visited[seed]) continue;
    agg_ids[seed] = n_agg;
    visited[seed] = 1;
    ++n_visited;
    int32_t size = 1;
    // candidates = sorted(adj[seed] - set(visited), key=degree)
    const SetEmu& so = adj[seed];
    SetEmu diff;
    if ((so.used >> 2) > n_visited) {
      diff = SetEmu::copy_of(so);
      so.for_each([&](int32_t k) {
        if (visited[k]) diff.discard(k);
      });
    } else {
      so.for_each([&](int32_t k) {
        if (!visited[k]) diff.add(k);
      });
    }
    cand.clear();
    diff.for_each([&](int32_t k) { cand.push_back(k); });
    std::stable_sort(cand.begin(), cand.end(),
                     [&](int32_t x, int32_t y) { return deg[x] < deg[y]; });
    for (int32_t nb : cand) {
      if (visited[nb]) continue;
      if (size >= max_agg_size) break;
      agg_ids[nb] = n_agg;
      visited[nb] = 1;
      ++n_visited;
      ++size;
      if (size < max_agg_size) {
        adj[nb].for_each([&](int32_t nb2) {
          if (!visited[nb2] && size < max_agg_size) {
            agg_ids[nb2] = n_agg;
            visited[nb2] = 1;
            ++n_visited;
            ++size;
          }
        });
      }
    }
    ++n_agg;
  }
  return n_agg;
}

// cons/tet_aggregation.py:145-211
void tet_hierarchy(const int32_t* t_i, int32_t nt, int32_t max_coarse, int32_t max_levels,
                   std::vector<int32_t>& sizes, std::vector<std::vector<int32_t>>& aggs) {
  sizes.assign(1, nt);
  aggs.clear();
  std::vector<int32_t> cur(t_i, t_i + 4LL * nt);
  int32_t cur_nt = nt;
  for (int32_t level = 0; level < max_levels; ++level) {
    if (cur_nt <= max_coarse) break;
    int32_t max_agg = std::min<int32_t>(8, std::max<int32_t>(2, cur_nt / std::max<int32_t>(max_coarse, 1)));
    max_agg = std::max<int32_t>(max_agg, 2);
    std::vector<int32_t> agg;
    int32_t n_agg = tet_aggregate(cur.data(), cur_nt, max_agg, agg);
    if (n_agg >= cur_nt) break;  // no coarsening progress (the level is popped)
    sizes.push_back(n_agg);
    aggs.push_back(agg);
    // virtual tets: aggregate a becomes (a, a, a, a)
    cur.assign(4LL * n_agg, 0);
    for (int32_t a = 0; a < n_agg; ++a)
      for (int l = 0; l < 4; ++l) cur[4LL * a + l] = a;
    cur_nt = n_agg;
  }
}

// ---------------------------------------------------------------------------
namespace {

struct Members {
  std::vector<int32_t> ptr, rows;  // fine rows of each aggregate, ascending
};

Members members_of(const int32_t* agg, int32_t n, int32_t n_agg) {
  Members m;
  m.ptr.assign(n_agg + 1, 0);
  for (int32_t i = 0; i < n; ++i) {
    if (agg[i] < 0 || agg[i] >= n_agg) throw std::invalid_argument("aggregate id out of range");
    m.ptr[agg[i] + 1]++;
  }
  for (int32_t a = 0; a < n_agg; ++a) m.ptr[a + 1] += m.ptr[a];
  m.rows.resize(n);
  std::vector<int32_t> cur(m.ptr.begin(), m.ptr.end() - 1);
  for (int32_t i = 0; i < n; ++i) m.rows[cur[agg[i]]++] = i;
  return m;
}

template <bool kByValue>
Galerkin galerkin_impl(const Csr& fine, const float* data, const int32_t* agg, int32_t n_agg) {
  const int32_t n = fine.n_rows;
  Members mem = members_of(agg, n, n_agg);
  Galerkin g;
  g.coarse.n_rows = g.coarse.n_cols = n_agg;
  std::vector<std::vector<int32_t>> rcols(n_agg), rmap(n_agg), rmapoff(n_agg);
#pragma omp parallel
  {
    std::vector<double> xs(kByValue ? n : 0, 0.0);
    std::vector<uint8_t> xt(n, 0);
    std::vector<int32_t> touched;
    std::vector<double> acc(kByValue ? n_agg : 0, 0.0);
    std::vector<int32_t> slot(n_agg, -1);
    std::vector<int32_t> jt;
    std::vector<std::vector<int32_t>> bucket;
#pragma omp for schedule(dynamic, 64)
    for (int32_t I = 0; I < n_agg; ++I) {
      touched.clear();
      // stage 1: X[I, j] = sum_{i in I ascending} A[i, j]
      for (int32_t m = mem.ptr[I]; m < mem.ptr[I + 1]; ++m) {
        int32_t i = mem.rows[m];
        for (int32_t k = fine.indptr[i]; k < fine.indptr[i + 1]; ++k) {
          int32_t j = fine.indices[k];
          if (!xt[j]) {
            xt[j] = 1;
            touched.push_back(j);
          }
          if (kByValue) xs[j] += static_cast<double>(data[k]);
        }
      }
      // stage 2: Ac[I, J] = sum_{j in J ascending} X[I, j]  (zeros dropped)
      std::sort(touched.begin(), touched.end());
      jt.clear();
      for (int32_t j : touched) {
        xt[j] = 0;
        if (kByValue) {
          double x = xs[j];
          xs[j] = 0.0;
          if (x == 0.0) continue;
          int32_t J = agg[j];
          if (slot[J] < 0) {
            slot[J] = 0;
            jt.push_back(J);
          }
          acc[J] += x;
        } else {
          int32_t J = agg[j];
          if (slot[J] < 0) {
            slot[J] = 0;
            jt.push_back(J);
          }
        }
      }
      std::sort(jt.begin(), jt.end());
      std::vector<int32_t>& cols = rcols[I];
      cols.clear();
      for (int32_t J : jt) {
        bool keep = true;
        if (kByValue) {
          keep = acc[J] != 0.0;
          acc[J] = 0.0;
        }
        slot[J] = -1;
        if (keep) cols.push_back(J);
      }
      // contribution map: for each kept (I, J), fine positions in
      // (member row ascending, stored position) order
      for (size_t c = 0; c < cols.size(); ++c) slot[cols[c]] = static_cast<int32_t>(c);
      if (bucket.size() < cols.size()) bucket.resize(cols.size());
      for (size_t c = 0; c < cols.size(); ++c) bucket[c].clear();
      for (int32_t m = mem.ptr[I]; m < mem.ptr[I + 1]; ++m) {
        int32_t i = mem.rows[m];
        for (int32_t k = fine.indptr[i]; k < fine.indptr[i + 1]; ++k) {
          int32_t s = slot[agg[fine.indices[k]]];
          if (s >= 0) bucket[s].push_back(k);
        }
      }
      std::vector<int32_t>& mp = rmap[I];
      std::vector<int32_t>& mo = rmapoff[I];
      mp.clear();
      mo.clear();
      for (size_t c = 0; c < cols.size(); ++c) {
        slot[cols[c]] = -1;
        mo.push_back(static_cast<int32_t>(bucket[c].size()));
        mp.insert(mp.end(), bucket[c].begin(), bucket[c].end());
      }
    }
  }
  g.coarse.indptr.assign(n_agg + 1, 0);
  int64_t nnz = 0, nmap = 0;
  for (int32_t I = 0; I < n_agg; ++I) {
    nnz += rcols[I].size();
    nmap += rmap[I].size();
    if (nnz > INT32_MAX || nmap > INT32_MAX) throw std::length_error("coarse nnz exceeds int32");
    g.coarse.indptr[I + 1] = static_cast<int32_t>(nnz);
  }
  g.coarse.indices.resize(nnz);
  g.contrib_idx.resize(nmap);
  g.contrib_off.assign(nnz + 1, 0);
  g.diag_pos.assign(n_agg, -1);
  int64_t pos = 0, mpos = 0;
  for (int32_t I = 0; I < n_agg; ++I) {
    for (size_t c = 0; c < rcols[I].size(); ++c) {
      g.coarse.indices[pos] = rcols[I][c];
      if (rcols[I][c] == I) g.diag_pos[I] = static_cast<int32_t>(pos);
      g.contrib_off[pos + 1] = g.contrib_off[pos] + rmapoff[I][c];
      ++pos;
    }
    std::copy(rmap[I].begin(), rmap[I].end(), g.contrib_idx.begin() + mpos);
    mpos += rmap[I].size();
  }
  return g;
}

}  // namespace

Galerkin galerkin(const Csr& fine, const float* data, const int32_t* agg_ids, int32_t n_agg) {
  return galerkin_impl<true>(fine, data, agg_ids, n_agg);
}

Galerkin galerkin_structural(const Csr& fine, const int32_t* agg_ids, int32_t n_agg) {
  return galerkin_impl<false>(fine, nullptr, agg_ids, n_agg);
}

// ---------------------------------------------------------------------------
int32_t graph_aggregate(const Csr& a, int32_t max_agg_size, std::vector<int32_t>& agg_ids) {
  const int32_t n = a.n_rows;
  agg_ids.assign(n, -1);
  int32_t n_agg = 0;
  // pass 1: a root whose neighbours are all free takes itself + neighbours
  for (int32_t i = 0; i < n; ++i) {
    if (agg_ids[i] >= 0) continue;
    bool free = true;
    for (int32_t k = a.indptr[i]; k < a.indptr[i + 1] && free; ++k)
      if (agg_ids[a.indices[k]] >= 0) free = false;
    if (!free) continue;
    int32_t size = 0;
    for (int32_t k = a.indptr[i]; k < a.indptr[i + 1] && size < max_agg_size; ++k) {
      int32_t j = a.indices[k];
      if (agg_ids[j] < 0) {
        agg_ids[j] = n_agg;
        ++size;
      }
    }
    if (agg_ids[i] < 0) agg_ids[i] = n_agg;
    ++n_agg;
  }
  // pass 2: leftovers join the neighbouring aggregate met first
  for (int32_t i = 0; i < n; ++i) {
    if (agg_ids[i] >= 0) continue;
    for (int32_t k = a.indptr[i]; k < a.indptr[i + 1]; ++k) {
      int32_t j = a.indices[k];
      if (j != i && agg_ids[j] >= 0) {
        agg_ids[i] = agg_ids[j];
        break;
      }
    }
    if (agg_ids[i] < 0) agg_ids[i] = n_agg++;
  }
  return n_agg;
}

// A slot repeating a vertex of an earlier slot of its constraint (a length
// constraint lists its edge twice) carries a zero gradient and is left out.
void vertex_incidence(const int32_t* t_i, int32_t nt, int32_t nv, std::vector<int32_t>& ptr,
                      std::vector<int32_t>& ent) {
  auto repeated = [&](int32_t t, int l) {
    for (int m = 0; m < l; ++m)
      if (t_i[4LL * t + m] == t_i[4LL * t + l]) return true;
    return false;
  };
  ptr.assign(nv + 1, 0);
  for (int32_t t = 0; t < nt; ++t)
    for (int l = 0; l < 4; ++l)
      if (!repeated(t, l)) ptr[t_i[4LL * t + l] + 1]++;
  for (int32_t v = 0; v < nv; ++v) ptr[v + 1] += ptr[v];
  ent.resize(ptr[nv]);
  std::vector<int32_t> cur(ptr.begin(), ptr.end() - 1);
  for (int32_t t = 0; t < nt; ++t)
    for (int l = 0; l < 4; ++l)
      if (!repeated(t, l)) ent[cur[t_i[4LL * t + l]]++] = 4 * t + l;
}

}  // namespace mgpbd
