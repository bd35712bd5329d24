// Boundary map: the reference's BoundaryCondition copy program, resolved once
// on the host into "which pre-BC slot does this slot hold after the BC".
//
// Every operation of BoundaryCondition (lbm.f90:96-155, lbm_3d.f90:96-157) is
// a copy within fb, including PassF with one periodic rank
// (cart_mpi.f90:240-277). Running that program, in the reference's serial
// order, on slot names instead of values gives for every slot the slot whose
// pre-BC value it ends up holding:
//   - a fluid slot  (this step's post-collision value),
//   - an obstacle (b_user) slot (the value it held before this BC, i.e. the
//     previous step's post-BC value),
//   - a solid slot that nothing ever writes (a constant),
//   - or "poison" when the chain reads outside the array, where the
//     reference's own value is undefined.
#pragma once

#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

namespace imx {

constexpr int64_t kPoison = -1;

struct GridLayout {
  int dim = 2, Q = 9;
  int L[3] = {1, 1, 1};  // local_length (interior nodes per dimension)
  int64_t dy = 0, dz = 0, N = 0;  // strides and padded cell count
  int e[81] = {};                 // lattice velocities, e[iq*dim+k]
  int64_t off(int iq, int mult) const {
    int64_t o = (int64_t)mult * e[iq * dim] + (int64_t)mult * dy * e[iq * dim + 1];
    if (dim == 3) o += (int64_t)mult * dz * e[iq * dim + 2];
    return o;
  }
  void coords(int64_t id, int& X, int& Y, int& Z) const {
    if (dim == 3) {
      Z = (int)(id / dz);
      id -= (int64_t)Z * dz;
    } else {
      Z = 0;
    }
    Y = (int)(id / dy);
    X = (int)(id - (int64_t)Y * dy);
  }
  bool is_ghost(int64_t id) const {
    int X, Y, Z;
    coords(id, X, Y, Z);
    if (X < 3 || X >= L[0] + 3 || Y < 3 || Y >= L[1] + 3) return true;
    return dim == 3 && (Z < 3 || Z >= L[2] + 3);
  }
  // Cell a ghost cell receives from in the one-rank periodic PassF.
  int64_t wrap_cell(int64_t id) const {
    int X, Y, Z;
    coords(id, X, Y, Z);
    auto w = [](int c, int l) { return c < 3 ? c + l : (c >= l + 3 ? c - l : c); };
    int64_t r = w(X, L[0]) + dy * w(Y, L[1]);
    if (dim == 3) r += dz * w(Z, L[2]);
    return r;
  }
};

// Kinds of a resolved source slot.
enum SrcKind : int { kSrcFluid = 0, kSrcUser = 1, kSrcStatic = 2, kSrcPoison = 3 };

struct BoundaryLists {
  const uint8_t* fluid_mask = nullptr;  // [N], 1 on nodes listed in fluid_id
  const int* bl = nullptr; int nl = 0;
  const int* br = nullptr; int nr = 0;
  const int* bu = nullptr; int nu = 0;
  const int* bd = nullptr; int nd = 0;
  const int* user = nullptr; int nuser = 0;
};

// One copy of the boundary program: after each collision, dst (a boundary
// slot in the freshly written buffer) takes the value of src; src_prev says
// that src is read from the other buffer (an obstacle slot's value before
// this BC). The fill kernel writes dst; with the copies inside the step
// kernel the puller of dst reads src instead. Slot indices are reference
// slots id*Q+iq.
struct FillEntry {
  int64_t dst;
  int64_t src;
  int src_prev;
};

class BoundaryMap {
 public:
  // Returns false with err set when the geometry is invalid.
  bool build(const GridLayout& g, const BoundaryLists& b, std::string& err);

  // Pre-BC slot that slot s holds after BoundaryCondition (kPoison if undefined).
  int64_t resolve(int64_t s) const;
  SrcKind kind_of(int64_t src) const;

  // The copies after each collision: every ghost slot some fluid node
  // pulls, plus every slot of every obstacle cell. Sorted by dst.
  const std::vector<FillEntry>& fill() const { return fill_; }
  // Interior obstacle cells (their slots carry values across iterations).
  const std::vector<int64_t>& user_cells() const { return user_cells_; }
  bool is_user_cell(int64_t id) const { return user_set_.count(id) != 0; }

 private:
  int64_t base(int64_t s) const;
  int64_t get(int64_t s) const;
  void set(int64_t s, int64_t v);

  GridLayout g_;
  const uint8_t* fluid_ = nullptr;
  std::unordered_map<int64_t, int64_t> cell_index_;  // written cell -> compact index
  std::vector<int64_t> names_;                        // compact*Q + iq -> name
  std::unordered_map<int64_t, int> user_set_;
  std::vector<int64_t> user_cells_;
  std::vector<FillEntry> fill_;
};

// ---------------------------------------------------------------------------
// The same program for a run on several MPI ranks (cart_mpi.f90): PassF
// gives every ghost cell of a rank the interior cell of the rank that owns
// its globally periodic position, and each rank then runs the copies on its
// own array. Names are (rank, slot) pairs, so a resolved source can live in
// another rank's buffer.

struct RankGeometry {
  GridLayout g;                          // the rank's local layout
  int start[3] = {0, 0, 0};              // local_start
  const uint8_t* fluid_mask = nullptr;   // [g.N]
  BoundaryLists lists;
};

struct GroupFillEntry {
  int64_t dst;       // slot id*Q+iq of the rank being filled
  int64_t src;       // slot in rank src_rank
  int src_rank;
  SrcKind kind;      // fluid / static: this step's buffer; user: the other one; poison
};

class GroupBoundary {
 public:
  // gl: global lengths n+1; np: ranks per dimension; ranks in MPI order.
  bool build(const std::vector<RankGeometry>& ranks, const int gl[3], const int np[3],
             std::string& err);
  // Rank a's refresh list after a collision (pipeline: ghost slots its
  // fluid nodes pull, every slot of its interior obstacle cells) or, with
  // complete, every ghost slot (download). Sorted by dst.
  bool fill(int a, bool complete, std::vector<GroupFillEntry>& out, std::string& err) const;

 private:
  static int64_t name(int rank, int64_t slot) { return ((int64_t)rank << 40) | slot; }
  static int rank_of(int64_t n) { return (int)(n >> 40); }
  static int64_t slot_of(int64_t n) { return n & ((int64_t(1) << 40) - 1); }
  int64_t base(int a, int64_t s) const;
  int64_t get(int a, int64_t s) const;
  SrcKind kind_of(int64_t n) const;

  struct Rank {
    RankGeometry geo;
    std::unordered_map<int64_t, int64_t> cell_index;  // written cell -> compact index
    std::vector<int64_t> names;
    std::unordered_map<int64_t, int> user_set;         // interior obstacle cells
    std::vector<int64_t> user_cells;
  };
  std::vector<Rank> r_;
  int gl_[3] = {1, 1, 1}, np_[3] = {1, 1, 1}, dim_ = 2;
};

}  // namespace imx
