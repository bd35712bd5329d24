// Boundary map construction (see bcmap.h).
#include "bcmap.h"

#include <algorithm>
#include <cstdio>

namespace imx {

int64_t BoundaryMap::base(int64_t s) const {
  const int64_t NQ = g_.N * g_.Q;
  if (s < 0 || s >= NQ) return kPoison;
  int64_t cell = s / g_.Q;
  int iq = (int)(s - cell * g_.Q);
  if (g_.is_ghost(cell)) return g_.wrap_cell(cell) * g_.Q + iq;  // PassF, one rank
  return s;
}

int64_t BoundaryMap::get(int64_t s) const {
  const int64_t NQ = g_.N * g_.Q;
  if (s < 0 || s >= NQ) return kPoison;
  int64_t cell = s / g_.Q;
  auto it = cell_index_.find(cell);
  if (it != cell_index_.end()) return names_[(size_t)(it->second * g_.Q + (s - cell * g_.Q))];
  return base(s);
}

void BoundaryMap::set(int64_t s, int64_t v) {
  int64_t cell = s / g_.Q;
  auto it = cell_index_.find(cell);
  names_[(size_t)(it->second * g_.Q + (s - cell * g_.Q))] = v;
}

int64_t BoundaryMap::resolve(int64_t s) const { return get(s); }

SrcKind BoundaryMap::kind_of(int64_t src) const {
  if (src == kPoison) return kSrcPoison;
  int64_t cell = src / g_.Q;
  if (fluid_[(size_t)cell]) return kSrcFluid;
  if (is_user_cell(cell)) return kSrcUser;
  return kSrcStatic;
}

bool BoundaryMap::build(const GridLayout& g, const BoundaryLists& b, std::string& err) {
  g_ = g;
  fluid_ = b.fluid_mask;
  cell_index_.clear();
  names_.clear();
  user_set_.clear();
  user_cells_.clear();
  fill_.clear();
  const int Q = g.Q;
  char msg[256];

  struct L { const int* p; int n; const char* name; };
  const L lists[5] = {{b.bu, b.nu, "bu"}, {b.bd, b.nd, "bd"}, {b.user, b.nuser, "b_user"},
                      {b.bl, b.nl, "bl"}, {b.br, b.nr, "br"}};
  for (const L& l : lists) {
    if (l.n < 0 || (l.n > 0 && !l.p)) {
      err = std::string("boundary list ") + l.name + " is missing";
      return false;
    }
    for (int i = 0; i < l.n; ++i) {
      int64_t id = l.p[i];
      if (id < 0 || id >= g.N) {
        snprintf(msg, sizeof msg, "%s[%d] = %lld is outside the padded array", l.name, i, (long long)id);
        err = msg;
        return false;
      }
      if (cell_index_.emplace(id, (int64_t)cell_index_.size()).second) {
        for (int iq = 0; iq < Q; ++iq) names_.push_back(base(id * Q + iq));
      }
    }
  }
  // Obstacle cells whose values persist from one iteration to the next: the
  // interior ones. (The reference's scan also visits the first ghost ring,
  // where the periodic geo halo can show a solid cell; such a ghost entry is
  // overwritten by PassF every iteration before the User loop writes it.)
  for (int i = 0; i < b.nuser; ++i) {
    int64_t id = b.user[i];
    if (fluid_[(size_t)id]) {
      snprintf(msg, sizeof msg, "b_user[%d] = %lld is a fluid node", i, (long long)id);
      err = msg;
      return false;
    }
    if (g.is_ghost(id)) continue;
    if (user_set_.emplace(id, (int)user_cells_.size()).second) user_cells_.push_back(id);
  }

  // The copy program, in the reference's serial order (lbm.f90:105-153).
  for (int l = 0; l < 3; ++l)  // Up, Down, User: fb(id,iq) = fb(id+2e_iq, nq-1-iq)
    for (int i = 0; i < lists[l].n; ++i) {
      int64_t id = lists[l].p[i];
      for (int iq = 0; iq < Q; ++iq) set(id * Q + iq, get((id + g.off(iq, 2)) * Q + (Q - 1 - iq)));
    }
  for (int i = 0; i < b.nl; ++i) {  // Inlet: fb(id,iq) = fb(id+1,iq)
    int64_t id = b.bl[i];
    for (int iq = 0; iq < Q; ++iq) set(id * Q + iq, get((id + 1) * Q + iq));
  }
  for (int i = 0; i < b.nr; ++i) {  // Outlet: fb(id,iq) = fb(id+e_iq,iq)
    int64_t id = b.br[i];
    for (int iq = 0; iq < Q; ++iq) set(id * Q + iq, get((id + g.off(iq, 1)) * Q + iq));
  }

  // Slots the copies after each collision must give a value.
  std::vector<int64_t> need;
  // (a) ghost slots pulled by a fluid node: ring-1 ghost cells (padded
  //     coordinates in [2, L+3], at least one on the rim).
  const int Zlo = g.dim == 3 ? 2 : 0, Zhi = g.dim == 3 ? g.L[2] + 3 : 0;
  for (int Z = Zlo; Z <= Zhi; ++Z)
    for (int Y = 2; Y <= g.L[1] + 3; ++Y)
      for (int X = 2; X <= g.L[0] + 3; ++X) {
        bool rim = X == 2 || X == g.L[0] + 3 || Y == 2 || Y == g.L[1] + 3 ||
                   (g.dim == 3 && (Z == 2 || Z == g.L[2] + 3));
        if (!rim) {
          X = g.L[0] + 2;  // jump to the far rim of this row
          continue;
        }
        int64_t c = X + g.dy * Y + g.dz * Z;
        for (int iq = 0; iq < Q; ++iq) {
          int64_t puller = c + g.off(iq, 1);
          if (puller >= 0 && puller < g.N && fluid_[(size_t)puller]) need.push_back(c * Q + iq);
        }
      }
  // (b) every slot of every obstacle cell (their values persist across steps).
  for (int64_t c : user_cells_)
    for (int iq = 0; iq < Q; ++iq) need.push_back(c * Q + iq);
  std::sort(need.begin(), need.end());
  need.erase(std::unique(need.begin(), need.end()), need.end());

  fill_.reserve(need.size());
  for (int64_t s : need) {
    int64_t r = get(s);
    SrcKind k = kind_of(r);
    if (k == kSrcPoison) {
      int X, Y, Z;
      g.coords(s / Q, X, Y, Z);
      snprintf(msg, sizeof msg,
               "boundary slot (x=%d,y=%d,z=%d,iq=%d) is filled from outside the array by the "
               "reference boundary program",
               X - 3, Y - 3, Z - 3, (int)(s % Q));
      err = msg;
      return false;
    }
    if (g.is_ghost(r / Q)) {
      err = "internal: boundary name resolved to a ghost slot";
      return false;
    }
    fill_.push_back(FillEntry{s, r, k == kSrcUser ? 1 : 0});
  }
  return true;
}

// ---------------------------------------------------------------------------
// GroupBoundary

int64_t GroupBoundary::base(int a, int64_t s) const {
  const Rank& R = r_[(size_t)a];
  const GridLayout& g = R.geo.g;
  if (s < 0 || s >= g.N * g.Q) return kPoison;
  const int64_t cell = s / g.Q;
  const int iq = (int)(s - cell * g.Q);
  if (!g.is_ghost(cell)) return name(a, s);
  // PassF: the owner of the globally periodic position
  int P[3];
  g.coords(cell, P[0], P[1], P[2]);
  int oc[3] = {0, 0, 0}, loc[3] = {3, 3, 3};
  for (int k = 0; k < dim_; ++k) {
    int gx = P[k] - 3 + R.geo.start[k];
    gx = ((gx % gl_[k]) + gl_[k]) % gl_[k];
    int q = 0, st = 0;
    for (;;) {
      const int len = gl_[k] / np_[k] + (q < gl_[k] % np_[k] ? 1 : 0);
      if (gx < st + len) break;
      st += len;
      ++q;
    }
    oc[k] = q;
    loc[k] = gx - st + 3;
  }
  const int b = dim_ == 2 ? oc[0] * np_[1] + oc[1] : (oc[0] * np_[1] + oc[1]) * np_[2] + oc[2];
  const GridLayout& o = r_[(size_t)b].geo.g;
  const int64_t oc_id = loc[0] + o.dy * loc[1] + (dim_ == 3 ? o.dz * loc[2] : 0);
  return name(b, oc_id * o.Q + iq);
}

int64_t GroupBoundary::get(int a, int64_t s) const {
  const Rank& R = r_[(size_t)a];
  const GridLayout& g = R.geo.g;
  if (s < 0 || s >= g.N * g.Q) return kPoison;
  const int64_t cell = s / g.Q;
  auto it = R.cell_index.find(cell);
  if (it != R.cell_index.end()) return R.names[(size_t)(it->second * g.Q + (s - cell * g.Q))];
  return base(a, s);
}

SrcKind GroupBoundary::kind_of(int64_t n) const {
  if (n == kPoison) return kSrcPoison;
  const Rank& R = r_[(size_t)rank_of(n)];
  const int64_t cell = slot_of(n) / R.geo.g.Q;
  if (R.geo.fluid_mask[(size_t)cell]) return kSrcFluid;
  if (R.user_set.count(cell)) return kSrcUser;
  return kSrcStatic;
}

bool GroupBoundary::build(const std::vector<RankGeometry>& ranks, const int gl[3], const int np[3],
                          std::string& err) {
  r_.clear();
  if (ranks.empty()) {
    err = "no ranks";
    return false;
  }
  dim_ = ranks[0].g.dim;
  for (int k = 0; k < 3; ++k) {
    gl_[k] = k < dim_ ? gl[k] : 1;
    np_[k] = k < dim_ ? np[k] : 1;
  }
  r_.resize(ranks.size());
  char msg[256];
  for (size_t a = 0; a < ranks.size(); ++a) r_[a].geo = ranks[a];
  // obstacle cells whose values persist: the interior ones of each rank
  for (size_t a = 0; a < ranks.size(); ++a) {
    Rank& R = r_[a];
    const BoundaryLists& b = R.geo.lists;
    for (int i = 0; i < b.nuser; ++i) {
      const int64_t id = b.user[i];
      if (id < 0 || id >= R.geo.g.N) {
        snprintf(msg, sizeof msg, "rank %d: b_user[%d] is outside the padded array", (int)a, i);
        err = msg;
        return false;
      }
      if (R.geo.fluid_mask[(size_t)id]) {
        snprintf(msg, sizeof msg, "rank %d: b_user[%d] = %lld is a fluid node", (int)a, i, (long long)id);
        err = msg;
        return false;
      }
      if (R.geo.g.is_ghost(id)) continue;
      if (R.user_set.emplace(id, (int)R.user_cells.size()).second) R.user_cells.push_back(id);
    }
  }
  // each rank's copy program on names, in the reference's serial order
  for (size_t a = 0; a < ranks.size(); ++a) {
    Rank& R = r_[a];
    const GridLayout& g = R.geo.g;
    const BoundaryLists& b = R.geo.lists;
    const int Q = g.Q;
    struct L { const int* p; int n; const char* name; };
    const L lists[5] = {{b.bu, b.nu, "bu"}, {b.bd, b.nd, "bd"}, {b.user, b.nuser, "b_user"},
                        {b.bl, b.nl, "bl"}, {b.br, b.nr, "br"}};
    for (const L& l : lists) {
      if (l.n < 0 || (l.n > 0 && !l.p)) {
        err = std::string("boundary list ") + l.name + " is missing";
        return false;
      }
      for (int i = 0; i < l.n; ++i) {
        const int64_t id = l.p[i];
        if (id < 0 || id >= g.N) {
          snprintf(msg, sizeof msg, "rank %d: %s[%d] is outside the padded array", (int)a, l.name, i);
          err = msg;
          return false;
        }
        if (R.cell_index.emplace(id, (int64_t)R.cell_index.size()).second)
          for (int iq = 0; iq < Q; ++iq) R.names.push_back(base((int)a, id * Q + iq));
      }
    }
    auto set = [&](int64_t s, int64_t v) {
      const int64_t cell = s / Q;
      R.names[(size_t)(R.cell_index[cell] * Q + (s - cell * Q))] = v;
    };
    for (int l = 0; l < 3; ++l)  // Up, Down, User: fb(id,iq) = fb(id+2e_iq, nq-1-iq)
      for (int i = 0; i < lists[l].n; ++i) {
        const int64_t id = lists[l].p[i];
        for (int iq = 0; iq < Q; ++iq)
          set(id * Q + iq, get((int)a, (id + g.off(iq, 2)) * Q + (Q - 1 - iq)));
      }
    for (int i = 0; i < b.nl; ++i) {  // Inlet: fb(id,iq) = fb(id+1,iq)
      const int64_t id = b.bl[i];
      for (int iq = 0; iq < Q; ++iq) set(id * Q + iq, get((int)a, (id + 1) * Q + iq));
    }
    for (int i = 0; i < b.nr; ++i) {  // Outlet: fb(id,iq) = fb(id+e_iq,iq)
      const int64_t id = b.br[i];
      for (int iq = 0; iq < Q; ++iq) set(id * Q + iq, get((int)a, (id + g.off(iq, 1)) * Q + iq));
    }
  }
  return true;
}

bool GroupBoundary::fill(int a, bool complete, std::vector<GroupFillEntry>& out,
                         std::string& err) const {
  out.clear();
  const Rank& R = r_[(size_t)a];
  const GridLayout& g = R.geo.g;
  const int Q = g.Q;
  std::vector<int64_t> need;
  if (complete) {
    const int PZ = g.dim == 3 ? g.L[2] + 6 : 1;
    for (int Z = 0; Z < PZ; ++Z)
      for (int Y = 0; Y < g.L[1] + 6; ++Y)
        for (int X = 0; X < g.L[0] + 6; ++X) {
          const int64_t c = X + g.dy * Y + g.dz * Z;
          if (!g.is_ghost(c)) continue;
          for (int iq = 0; iq < Q; ++iq) need.push_back(c * Q + iq);
        }
  } else {
    // ring-1 ghost slots pulled by a fluid node, and every obstacle slot
    const int Zlo = g.dim == 3 ? 2 : 0, Zhi = g.dim == 3 ? g.L[2] + 3 : 0;
    for (int Z = Zlo; Z <= Zhi; ++Z)
      for (int Y = 2; Y <= g.L[1] + 3; ++Y)
        for (int X = 2; X <= g.L[0] + 3; ++X) {
          const bool rim = X == 2 || X == g.L[0] + 3 || Y == 2 || Y == g.L[1] + 3 ||
                           (g.dim == 3 && (Z == 2 || Z == g.L[2] + 3));
          if (!rim) continue;
          const int64_t c = X + g.dy * Y + g.dz * Z;
          for (int iq = 0; iq < Q; ++iq) {
            const int64_t puller = c + g.off(iq, 1);
            if (puller >= 0 && puller < g.N && R.geo.fluid_mask[(size_t)puller]) need.push_back(c * Q + iq);
          }
        }
    for (int64_t c : R.user_cells)
      for (int iq = 0; iq < Q; ++iq) need.push_back(c * Q + iq);
  }
  std::sort(need.begin(), need.end());
  need.erase(std::unique(need.begin(), need.end()), need.end());
  out.reserve(need.size());
  char msg[256];
  for (int64_t s : need) {
    const int64_t n = get(a, s);
    const SrcKind k = kind_of(n);
    if (k == kSrcPoison) {
      if (complete) {
        out.push_back(GroupFillEntry{s, 0, a, kSrcPoison});
        continue;
      }
      int X, Y, Z;
      g.coords(s / Q, X, Y, Z);
      snprintf(msg, sizeof msg,
               "rank %d: boundary slot (x=%d,y=%d,z=%d,iq=%d) is filled from outside the array by "
               "the reference boundary program",
               a, X - 3 + R.geo.start[0], Y - 3 + R.geo.start[1], Z - 3 + R.geo.start[2], (int)(s % Q));
      err = msg;
      return false;
    }
    const Rank& O = r_[(size_t)rank_of(n)];
    if (O.geo.g.is_ghost(slot_of(n) / O.geo.g.Q)) {
      err = "internal: group boundary name resolved to a ghost slot";
      return false;
    }
    out.push_back(GroupFillEntry{s, slot_of(n), rank_of(n), k});
  }
  return true;
}

}  // namespace imx
