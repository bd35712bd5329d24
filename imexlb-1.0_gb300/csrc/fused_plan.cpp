// Host side of the fused boundary copies (fused_plan.h).
#include "fused_plan.h"

#include <algorithm>
#include <unordered_map>

namespace imx {

int64_t fused_form(const GridLayout& gl, const DevGrid& g, int64_t pshift, int64_t p,
                   uint32_t bits, int q) {
  const int dim = gl.dim, Q = gl.Q;
  const int64_t N = gl.N;
  const int ex = gl.e[q * dim], ey = gl.e[q * dim + 1], ez = dim == 3 ? gl.e[q * dim + 2] : 0;
  const int ew = dim == 3 ? ez : ey;
  const bool opp = (ew == 1 && (bits & kMaskWallLo)) || (ew == -1 && (bits & kMaskWallHi));
  int64_t a = opp ? (int64_t)(Q - 1 - q) * N + p + g.off[q] : (int64_t)q * N + p - g.off[q];
  if (ex == 1 && (bits & kMaskInlet)) a += 1;
  if (ex == -1 && (bits & kMaskOutlet)) a += g.off[q];
  if (dim == 3 && ey == 1 && (bits & kMaskPerLo)) a += pshift;
  if (dim == 3 && ey == -1 && (bits & kMaskPerHi)) a -= pshift;
  return a;
}

void fused_kind_offsets(const GridLayout& gl, const DevGrid& g, int64_t pshift,
                        std::vector<int64_t>& out) {
  const int Q = gl.Q;
  out.assign((size_t)27 * Q, 0);
  for (int k = 0; k < 27; ++k) {
    const int x = k % 3, w = (k / 3) % 3, y = k / 9;
    uint32_t bits = 0;
    if (x == 1) bits |= kMaskInlet;
    if (x == 2) bits |= kMaskOutlet;
    if (w == 1) bits |= kMaskWallLo;
    if (w == 2) bits |= kMaskWallHi;
    if (y == 1) bits |= kMaskPerLo;
    if (y == 2) bits |= kMaskPerHi;
    for (int q = 0; q < Q; ++q)
      out[(size_t)k * Q + q] = (int64_t)q * gl.N - fused_form(gl, g, pshift, 0, bits, q);
  }
}

bool plan_fused(const GridLayout& gl, const DevGrid& g, const std::vector<uint8_t>& mask,
                const BoundaryMap& bmap, const std::vector<DevFill>& fill, FusedPlan& out) {
  out = FusedPlan{};
  const int Q = gl.Q, dim = gl.dim;
  const int64_t N = gl.N;
  out.pshift = dim == 3 ? (int64_t)gl.L[1] * gl.dy : 0;
  auto fluid = [&](int64_t c) {
    return c >= g.id_lo && c < g.id_hi && (mask[(size_t)c] & kMaskFluid) != 0;
  };
  auto nearest_fluid = [&](int64_t c) -> int64_t {
    for (int64_t d = 1; d < N; ++d) {
      if (fluid(c + d)) return c + d;
      if (fluid(c - d)) return c - d;
      if (c + d >= g.id_hi && c - d < g.id_lo) break;
    }
    return -1;
  };
  // ghost copies become redirects of the node that pulls them; obstacle
  // copies run in the node that writes their source
  std::unordered_map<int64_t, std::vector<std::pair<int, uint32_t>>> rim;
  struct P { int64_t x; DevFill32 e; };
  std::vector<P> push;
  for (const DevFill& e : fill) {
    if (e.src == kFillNaN) return false;
    const int64_t dc = e.dst % N;
    const int dq = (int)(e.dst / N);
    if (gl.is_ghost(dc)) {
      const int64_t p = dc + g.off[dq];
      if (e.src < 0 || !fluid(p)) return false;
      rim[p].push_back({dq, (uint32_t)e.src});
    } else if (bmap.is_user_cell(dc)) {
      int64_t x = -1;
      if (e.src >= 0 && fluid(e.src % N)) {
        x = e.src % N;
      } else {
        const int64_t puller = dc + g.off[dq];
        x = fluid(puller) ? puller : nearest_fluid(dc);
        if (x < 0) return false;
      }
      push.push_back(P{x, DevFill32{(uint32_t)e.dst, (int32_t)e.src}});
    } else {
      return false;
    }
  }
  // candidates: every node that pulls from the rim, and every inlet / outlet
  // node (their bits select closed forms on the device)
  std::vector<int64_t> cand;
  for (const auto& kv : rim) cand.push_back(kv.first);
  for (int64_t c = g.id_lo; c < g.id_hi; ++c)
    if (fluid(c) && (mask[(size_t)c] & (kMaskInlet | kMaskOutlet)) && !rim.count(c)) cand.push_back(c);
  std::sort(cand.begin(), cand.end());
  std::vector<int64_t> table;
  std::vector<int64_t> want((size_t)Q);
  const int wax = dim == 3 ? 2 : 1;
  for (int64_t p : cand) {
    int X, Y, Z;
    gl.coords(p, X, Y, Z);
    const int W = dim == 3 ? Z : Y;
    uint32_t F = mask[(size_t)p] & (kMaskInlet | kMaskOutlet);
    if (W == 3) F |= kMaskWallLo;
    if (W == gl.L[wax] + 2) F |= kMaskWallHi;
    if (dim == 3 && Y == 3) F |= kMaskPerLo;
    if (dim == 3 && Y == gl.L[1] + 2) F |= kMaskPerHi;
    for (int q = 0; q < Q; ++q) want[(size_t)q] = (int64_t)q * N + p - g.off[q];
    auto it = rim.find(p);
    if (it != rim.end())
      for (const auto& qr : it->second) want[(size_t)qr.first] = qr.second;
    // one table per kind: both faces of a pair (a one-node-wide lattice) go
    // to a record
    bool closed = !((F & kMaskInlet) && (F & kMaskOutlet)) && !((F & kMaskWallLo) && (F & kMaskWallHi)) &&
                  !((F & kMaskPerLo) && (F & kMaskPerHi));
    for (int q = 0; q < Q && closed; ++q) closed = fused_form(gl, g, out.pshift, p, F, q) == want[(size_t)q];
    if (closed) {
      const uint8_t b = (uint8_t)(F & ~(uint32_t)(kMaskInlet | kMaskOutlet));
      if (b) out.face.push_back({p, b});
    } else {
      table.push_back(p);
    }
  }
  // one record per row node and per node that runs obstacle copies; a
  // record replaces the closed forms, so its row lists every rim source
  std::sort(push.begin(), push.end(), [](const P& a, const P& b) {
    return a.x != b.x ? a.x < b.x : a.e.dst < b.e.dst;
  });
  out.nodes = table;
  for (const P& x : push) out.nodes.push_back(x.x);
  std::sort(out.nodes.begin(), out.nodes.end());
  out.nodes.erase(std::unique(out.nodes.begin(), out.nodes.end()), out.nodes.end());
  std::unordered_map<int64_t, size_t> rec_of;
  out.rec.assign(out.nodes.size() * (size_t)(Q + 1), kNoRedirect);
  for (size_t k = 0; k < out.nodes.size(); ++k) {
    rec_of[out.nodes[k]] = k;
    out.rec[k * (Q + 1) + Q] = 0u;  // no obstacle copies
    auto it = rim.find(out.nodes[k]);
    if (it != rim.end())
      for (const auto& qr : it->second) out.rec[k * (Q + 1) + qr.first] = qr.second;
  }
  if (push.size() >= (size_t(1) << 24)) return false;
  out.ent.resize(push.size());
  for (size_t i = 0; i < push.size();) {
    size_t j = i;
    while (j < push.size() && push[j].x == push[i].x) {
      out.ent[j] = push[j].e;
      ++j;
    }
    if (j - i > 255) return false;
    out.rec[rec_of[push[i].x] * (size_t)(Q + 1) + Q] = (uint32_t)(i << 8) | (uint32_t)(j - i);
    i = j;
  }
  // record nodes drop their closed forms
  out.face.erase(std::remove_if(out.face.begin(), out.face.end(),
                                [&](const std::pair<int64_t, uint8_t>& f) { return rec_of.count(f.first) != 0; }),
                 out.face.end());
  return true;
}

void apply_plan_bits(const FusedPlan& p, std::vector<uint8_t>& mask) {
  for (const auto& f : p.face) mask[(size_t)f.first] |= f.second;
  for (int64_t x : p.nodes) mask[(size_t)x] |= kMaskRecord;
}

}  // namespace imx
