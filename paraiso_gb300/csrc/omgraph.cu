// omgraph.cu -- Orthotope Machine graphs compiled into GB300 kernels at run
// time.  The reference's generator lowers an OM graph to a plan of
// sub-kernels and prints C++/CUDA for them
// (Language/Paraiso/Generator/OMTrans.hs:39-56, PlanTrans.hs:282-596).  Here
// the graph arrives as text (the format of paraiso_gb300/omgraph.py), and
// each OM kernel becomes a few CUDA kernels generated as source and compiled
// with NVRTC for sm_103a:
//   * one "stage" per reduce depth: a grid-stride pass over the memory array
//     that writes every array store of that depth (its value on its valid
//     region, zero elsewhere, into the static's other buffer) and folds every
//     reduce of that depth into per-block partials; the last block combines
//     the partials in a fixed order;
//   * one "commit" thread that evaluates the scalar stores.
// Values other than stores and reduces are recomputed where they are used
// (the generator's Delayed allocation), once per (node, offset) per cell,
// except that a stage which reads a computed value at three or more offsets
// computes it once per cell of a shared-memory tile (plan_tiles).
// Semantics followed: valid regions (Optimization/BoundaryAnalysis.hs:33-94),
// margins (OMTrans.hs:103-120), shift reads x[c - v] (PlanTrans.hs:561-562),
// loadIndex / loadSize (PlanTrans.hs:455-466), Arith -> C (PlanTrans.hs:
// 670-710), statics updated when the kernel ends (PlanTrans.hs:243-258).
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "om_internal.cuh"

namespace om {
namespace og {

enum Type { TInt = 0, TFloat, TDouble, TBool };

static const char *ctype(Type t) {
  switch (t) {
    case TInt: return "int";
    case TFloat: return "float";
    case TDouble: return "double";
    default: return "bool";
  }
}
static int tsize(Type t) { return t == TDouble ? 8 : (t == TBool ? 1 : 4); }

struct Node {
  int id = -1;
  std::string op;
  bool array = true;
  Type type = TInt;
  std::vector<int> args;  // operand node ids
  std::string sarg;       // static name, reduce operator or literal
  int vec[2] = {0, 0};    // shift vector or axis
};

struct Store {
  int stat;
  int node;
};

struct KernelDef {
  std::string name;
  std::vector<Node> nodes;
  std::map<int, int> at;  // node id -> index in nodes
  std::vector<Store> stores;
  std::set<int> manifest;  // array nodes marked Manifest (stored once per run)
  const Node &node(int id) const { return nodes[at.at(id)]; }
};

struct StaticDef {
  std::string name;
  bool array;
  Type type;
  size_t offset = 0;  // scalar: byte offset in the scalar block
};

struct Graph {
  std::string name;
  int ndim = 2;
  int size[2] = {1, 1};
  bool open = false;
  std::vector<StaticDef> statics;
  std::vector<KernelDef> kernels;
  int find_static(const std::string &n) const {
    for (size_t i = 0; i < statics.size(); ++i)
      if (statics[i].name == n) return (int)i;
    return -1;
  }
};

// ---------------------------------------------------------------------------
// parsing
// ---------------------------------------------------------------------------

static bool parse_type(const std::string &s, Type *t) {
  if (s == "int") *t = TInt;
  else if (s == "float") *t = TFloat;
  else if (s == "double") *t = TDouble;
  else if (s == "bool") *t = TBool;
  else return false;
  return true;
}

static const char *kArith[] = {"add", "sub", "mul", "div", "mod", "neg", "inv", "not",
                               "and", "or", "eq", "ne", "lt", "le", "gt", "ge",
                               "select", "max", "min", "abs", "signum", "sqrt", "exp",
                               "log", "sin", "cos", "tan", "asin", "acos", "atan",
                               "atan2", "pow", "cast"};

static int arity(const std::string &op) {
  static const char *one[] = {"neg", "inv", "not", "abs", "signum", "sqrt", "exp", "log",
                              "sin", "cos", "tan", "asin", "acos", "atan", "cast"};
  for (const char *o : one)
    if (op == o) return 1;
  if (op == "select") return 3;
  return 2;
}

static bool is_arith(const std::string &op) {
  for (const char *o : kArith)
    if (op == o) return true;
  return false;
}

static om_status perr(int line, const std::string &what) {
  set_error("om_create_graph: line " + std::to_string(line) + ": " + what);
  return OM_ERR_ARG;
}

// Structurally equal nodes (same operation, realm, type, literal or static,
// vector and operands) compute the same value: keep the first of each class
// and point every use at it.  The Haskell builder makes a new node for each
// application of a function, so a graph such as examples/Hydro repeats
// literals, comparisons and whole expressions.  Merged, the field selects of
// one HLLC wall record share their condition, which lets the emitter branch
// on it once for the whole record.  A class is Manifest if any member was.
static void merge_duplicates(KernelDef &k) {
  std::map<std::string, int> first;
  std::map<int, int> rep;
  std::vector<Node> kept;
  std::map<int, int> at;
  for (Node n : k.nodes) {
    for (int &a : n.args) a = rep.at(a);
    std::ostringstream key;
    key << n.op << '|' << n.array << '|' << (int)n.type << '|' << n.sarg << '|' << n.vec[0] << '|'
        << n.vec[1];
    for (int a : n.args) key << '|' << a;
    const auto it = first.find(key.str());
    if (it != first.end()) {
      rep[n.id] = it->second;
      continue;
    }
    first[key.str()] = n.id;
    rep[n.id] = n.id;
    at[n.id] = (int)kept.size();
    kept.push_back(n);
  }
  for (Store &st : k.stores) st.node = rep.at(st.node);
  std::set<int> man;
  for (int m : k.manifest) man.insert(rep.at(m));
  k.nodes = kept;
  k.at = at;
  k.manifest = man;
}

static om_status parse(const char *text, Graph *g) {
  std::istringstream in(text);
  std::string l;
  int ln = 0;
  KernelDef *k = nullptr;
  bool head = false;
  while (std::getline(in, l)) {
    ++ln;
    std::istringstream ws(l);
    std::vector<std::string> w;
    for (std::string t; ws >> t;) w.push_back(t);
    if (w.empty() || w[0][0] == '#') continue;
    if (!head) {
      if (w[0] != "om" || w.size() < 4) return perr(ln, "expected 'om NAME NDIM SIZES BOUNDARY'");
      g->name = w[1];
      g->ndim = std::atoi(w[2].c_str());
      if (g->ndim < 1 || g->ndim > 2 || (int)w.size() != 4 + g->ndim)
        return perr(ln, "1 or 2 dimensions");
      for (int a = 0; a < g->ndim; ++a) {
        g->size[a] = std::atoi(w[3 + a].c_str());
        if (g->size[a] < 1 || g->size[a] > (1 << 20)) return perr(ln, "size out of range");
      }
      const std::string &b = w[3 + g->ndim];
      if (b != "cyclic" && b != "open") return perr(ln, "boundary cyclic or open");
      g->open = b == "open";
      head = true;
      continue;
    }
    if (w[0] == "static") {
      if (k || w.size() != 4) return perr(ln, "static NAME array|scalar TYPE");
      StaticDef s;
      s.name = w[1];
      if (w[2] != "array" && w[2] != "scalar") return perr(ln, "realm array or scalar");
      s.array = w[2] == "array";
      if (!parse_type(w[3], &s.type)) return perr(ln, "unknown type " + w[3]);
      if (g->find_static(s.name) >= 0) return perr(ln, "duplicate static " + s.name);
      g->statics.push_back(s);
      continue;
    }
    if (w[0] == "kernel") {
      if (k || w.size() != 2) return perr(ln, "kernel NAME (inside no other kernel)");
      g->kernels.push_back(KernelDef());
      k = &g->kernels.back();
      k->name = w[1];
      continue;
    }
    if (w[0] == "end") {
      if (!k) return perr(ln, "end outside a kernel");
      merge_duplicates(*k);
      k = nullptr;
      continue;
    }
    if (!k) return perr(ln, "node outside a kernel");
    if (w[0] == "store") {
      if (w.size() != 3) return perr(ln, "store STATIC NODE");
      const int s = g->find_static(w[1]);
      const int id = std::atoi(w[2].c_str());
      if (s < 0) return perr(ln, "no static " + w[1]);
      if (!k->at.count(id)) return perr(ln, "unknown node " + w[2]);
      const Node &v = k->node(id);
      if (v.array != g->statics[s].array || v.type != g->statics[s].type)
        return perr(ln, "store of a value whose realm or type differs from " + w[1]);
      k->stores.push_back(Store{s, id});
      continue;
    }
    if (w[0] == "manifest") {
      if (w.size() != 2) return perr(ln, "manifest NODE");
      const int id = std::atoi(w[1].c_str());
      if (!k->at.count(id)) return perr(ln, "unknown node " + w[1]);
      if (!k->node(id).array) return perr(ln, "manifest of an array node");
      k->manifest.insert(id);
      continue;
    }
    if (w.size() < 4) return perr(ln, "ID OP REALM TYPE ...");
    Node n;
    n.id = std::atoi(w[0].c_str());
    n.op = w[1];
    if (w[2] != "array" && w[2] != "scalar") return perr(ln, "realm array or scalar");
    n.array = w[2] == "array";
    if (!parse_type(w[3], &n.type)) return perr(ln, "unknown type " + w[3]);
    if (k->at.count(n.id)) return perr(ln, "duplicate node id");
    auto node_arg = [&](size_t i, int *out) -> bool {
      if (i >= w.size()) return false;
      const int id = std::atoi(w[i].c_str());
      if (!k->at.count(id)) return false;
      *out = id;
      return true;
    };
    if (n.op == "load") {
      if (w.size() != 5) return perr(ln, "load STATIC");
      const int s = g->find_static(w[4]);
      if (s < 0) return perr(ln, "no static " + w[4]);
      if (g->statics[s].array != n.array || g->statics[s].type != n.type)
        return perr(ln, "load realm/type differs from the static");
      n.sarg = w[4];
    } else if (n.op == "imm") {
      if (w.size() != 5) return perr(ln, "imm LITERAL");
      n.sarg = w[4];
    } else if (n.op == "shift") {
      if ((int)w.size() != 5 + g->ndim || !n.array) return perr(ln, "shift NODE V0 [V1]");
      int a;
      if (!node_arg(4, &a) || !k->node(a).array) return perr(ln, "shift of an array node");
      n.args.push_back(a);
      for (int d = 0; d < g->ndim; ++d) n.vec[d] = std::atoi(w[5 + d].c_str());
      if (k->node(a).type != n.type) return perr(ln, "shift keeps the type");
    } else if (n.op == "loadindex" || n.op == "loadsize") {
      if (w.size() != 5) return perr(ln, n.op + " AXIS");
      n.vec[0] = std::atoi(w[4].c_str());
      if (n.vec[0] < 0 || n.vec[0] >= g->ndim) return perr(ln, "axis out of range");
      if (n.type != TInt || n.array != (n.op == "loadindex"))
        return perr(ln, "loadindex is an int array, loadsize an int scalar");
    } else if (n.op == "reduce") {
      if (w.size() != 6 || n.array) return perr(ln, "reduce OP NODE (a scalar)");
      n.sarg = w[4];
      if (n.sarg != "sum" && n.sarg != "min" && n.sarg != "max")
        return perr(ln, "reduce sum|min|max");
      int a;
      if (!node_arg(5, &a) || !k->node(a).array || k->node(a).type != n.type ||
          n.type == TBool)
        return perr(ln, "reduce of a numeric array node of the same type");
      n.args.push_back(a);
    } else if (n.op == "broadcast") {
      int a;
      if (w.size() != 5 || !n.array || !node_arg(4, &a) || k->node(a).array ||
          k->node(a).type != n.type)
        return perr(ln, "broadcast of a scalar node of the same type");
      n.args.push_back(a);
    } else if (is_arith(n.op)) {
      const int ar = arity(n.op);
      if ((int)w.size() != 4 + ar) return perr(ln, n.op + " takes " + std::to_string(ar));
      for (int i = 0; i < ar; ++i) {
        int a;
        if (!node_arg(4 + i, &a)) return perr(ln, "unknown operand");
        if (k->node(a).array != n.array) return perr(ln, "operand realm differs");
        n.args.push_back(a);
      }
      if (n.op == "mod" && n.type != TInt) return perr(ln, "mod of int values");
    } else {
      return perr(ln, "unknown operation " + n.op);
    }
    k->at[n.id] = (int)k->nodes.size();
    k->nodes.push_back(n);
  }
  if (!head) return perr(ln, "empty graph");
  if (k) return perr(ln, "kernel without end");
  return OM_OK;
}

// ---------------------------------------------------------------------------
// valid regions and margins
// ---------------------------------------------------------------------------

struct Iv {
  bool lo_inf = true, hi_inf = true;
  int lo = 0, hi = 0;  // offsets from the lower / upper edge of the array
};
struct Region {
  Iv ax[2];
};

static Region full_region() {
  Region r;
  for (auto &a : r.ax) { a.lo_inf = a.hi_inf = false; a.lo = a.hi = 0; }
  return r;
}

static Region meet(const Region &a, const Region &b) {
  Region r;
  for (int d = 0; d < 2; ++d) {
    const Iv &x = a.ax[d], &y = b.ax[d];
    Iv &z = r.ax[d];
    z.lo_inf = x.lo_inf && y.lo_inf;
    z.lo = x.lo_inf ? y.lo : (y.lo_inf ? x.lo : std::max(x.lo, y.lo));
    z.hi_inf = x.hi_inf && y.hi_inf;
    z.hi = x.hi_inf ? y.hi : (y.hi_inf ? x.hi : std::min(x.hi, y.hi));
  }
  return r;
}

static std::vector<Region> regions(const KernelDef &k) {
  std::vector<Region> reg(k.nodes.size());
  for (size_t i = 0; i < k.nodes.size(); ++i) {
    const Node &n = k.nodes[i];
    if (!n.array || n.op == "imm" || n.op == "loadindex" || n.op == "broadcast") {
      reg[i] = Region();
    } else if (n.op == "load") {
      reg[i] = full_region();
    } else if (n.op == "shift") {
      Region m = reg[k.at.at(n.args[0])];
      for (int d = 0; d < 2; ++d) {
        m.ax[d].lo += n.vec[d];
        m.ax[d].hi += n.vec[d];
      }
      reg[i] = meet(m, full_region());
    } else {
      Region r;
      for (int a : n.args) r = meet(r, reg[k.at.at(a)]);
      reg[i] = r;
    }
  }
  return reg;
}

// ---------------------------------------------------------------------------
// code generation
// ---------------------------------------------------------------------------

struct Layout {
  int ms[2];
  int lm[2];
  bool open;
  int size[2];
};

static std::string lit(Type t, const std::string &s) {
  if (t == TBool) return (s == "0" || s == "false") ? "false" : "true";
  if (t == TInt) return "(" + std::to_string(std::strtoll(s.c_str(), nullptr, 10)) + ")";
  const double v = std::strtod(s.c_str(), nullptr);
  if (v != v) return t == TFloat ? "(om_inf_f() - om_inf_f())" : "(om_inf_d() - om_inf_d())";
  if (v == 1.0 / 0.0) return t == TFloat ? "om_inf_f()" : "om_inf_d()";
  if (v == -1.0 / 0.0) return t == TFloat ? "(-om_inf_f())" : "(-om_inf_d())";
  char buf[64];
  std::snprintf(buf, sizeof buf, "%a", v);
  return t == TFloat ? std::string("((float)") + buf + ")" : std::string("(") + buf + ")";
}

// A stage whose per-cell code has at most kMaxVectorStatements statements
// evaluates kCellsPerThread cells per thread (eight per thread measured
// slower on the Life graph: 233 against 364 Gcell-updates/s).
constexpr int kCellsPerThread = 4;
constexpr int kMaxVectorStatements = 400;

// Emits the statements computing (node, offset) values of one kernel, each
// once, into a block of code.
// Where the manifests of a kernel are: node id -> {stage that computes it,
// its array among the handle's temporaries}.
struct ManifestAt {
  int stage;
  int tmp;
};

// A value computed once per cell of a stage's shared-memory tile (with its
// halo) and read there at every offset the stage needs it: node id -> the
// tile array.
struct TileAt {
  std::string name;
};

// The tile of a tiled stage: TX x TY cells per block, a halo of hx0/hy0
// cells below and hx1/hy1 above each axis; RX x RY cells in all.
struct TileShape {
  int tx = 32, ty = 8, hx0 = 0, hx1 = 0, hy0 = 0, hy1 = 0;
  int rx() const { return tx + hx0 + hx1; }
  int ry() const { return ty + hy0 + hy1; }
};

class Emitter {
 public:
  Emitter(const Graph &g, const KernelDef &k, const Layout &L,
          const std::map<int, int> &slot_of_reduce,
          const std::map<int, ManifestAt> *manifests = nullptr, int stage = 0)
      : g_(g), k_(k), L_(L), slots_(slot_of_reduce), man_(manifests), stage_(stage) {
    for (const Node &n : k.nodes)
      if (n.op == "select" && n.array) groups_[n.args[0]].push_back(n.id);
  }

  std::string code;

  std::string value(int id, int o0, int o1) {
    const Node &n = k_.node(id);
    if (!n.array) o0 = o1 = 0;
    const auto key = std::make_tuple(id, o0, o1);
    auto it = memo_.find(key);
    if (it != memo_.end()) return it->second;
    std::string expr;
    const std::string T = ctype(n.type);
    if (tiles_ && tiles_->count(id)) {
      // computed by the tile phase of this stage, for every cell of the tile
      const std::string v = "t" + std::to_string(id) + "_" + off_name(o0) + "_" + off_name(o1);
      code += "      const " + T + " " + v + " = " + tiles_->at(id).name + "[(ty + " +
              std::to_string(o1 + shape_.hy0) + ") * " + std::to_string(shape_.rx()) + " + tx + " +
              std::to_string(o0 + shape_.hx0) + "];\n";
      return memo_[key] = v;
    }
    const ManifestAt *m = nullptr;
    if (man_) {
      auto mi = man_->find(id);
      if (mi != man_->end() && mi->second.stage < stage_) m = &mi->second;
    }
    if (m) {
      // a manifest computed by an earlier stage of this kernel run
      expr = element("P.tmp[" + std::to_string(m->tmp) + "]", n.type, o0, o1);
    } else if (n.op == "load") {
      const int s = g_.find_static(n.sarg);
      if (g_.statics[s].array)
        expr = element("P.cur[" + std::to_string(array_index(s)) + "]", n.type, o0, o1);
      else
        expr = scalar_read(g_.statics[s]);
    } else if (n.op == "imm") {
      expr = lit(n.type, n.sarg);
    } else if (n.op == "shift") {
      return memo_[key] = value(n.args[0], o0 - n.vec[0], o1 - n.vec[1]);
    } else if (n.op == "loadindex") {
      const int ax = n.vec[0];
      const std::string c = ax == 0 ? "c0" : "c1";
      const int off = (ax == 0 ? o0 : o1) - L_.lm[ax];
      if (L_.open)
        expr = "(" + c + " + (" + std::to_string(off) + "))";
      else
        expr = wrap(c, ax == 0 ? o0 : o1, L_.ms[ax]);
    } else if (n.op == "loadsize") {
      expr = std::to_string(g_.size[n.vec[0]]);
    } else if (n.op == "reduce") {
      expr = "(*(const " + T + " *)(slots + " + std::to_string(8 * slots_.at(id)) + "))";
    } else if (n.op == "broadcast") {
      return memo_[key] = value(n.args[0], 0, 0);
    } else if (n.op == "select" && lazy_ && n.array &&
               !open_.count(std::make_tuple(n.args[0], o0, o1))) {
      select_group(n.args[0], o0, o1);
      return memo_.at(key);
    } else {
      std::vector<std::string> a;
      for (int x : n.args) a.push_back(value(x, o0, o1));
      expr = arith(n, a);
    }
    const std::string v = "v" + std::to_string(id) + "_" + off_name(o0) + "_" + off_name(o1);
    code += "      const " + T + " " + v + " = " + expr + ";\n";
    return memo_[key] = v;
  }

  int array_index(int s) const {
    int k = 0;
    for (int i = 0; i < s; ++i) k += g_.statics[i].array ? 1 : 0;
    return k;
  }

  // Branch on a select's condition instead of computing both operands:
  // every array select with that condition (the fields of one record) is
  // assigned in one if/else, each side computing only its operands.  Values
  // first computed inside a side stay there (the memo is restored after
  // it), so the arithmetic of every value is unchanged.  Not for four cells
  // per thread, whose shuffles need the whole warp.
  void lazy_selects(bool on) { lazy_ = on; }

  // values that a tile phase computes, read from its tile (phase two of a
  // tiled stage)
  void tiled(const std::map<int, TileAt> *t, const TileShape &shape) {
    tiles_ = t;
    shape_ = shape;
  }

  // the offsets at which each node has been evaluated so far
  std::map<int, std::set<std::pair<int, int>>> offsets() const {
    std::map<int, std::set<std::pair<int, int>>> r;
    for (const auto &m : memo_) r[std::get<0>(m.first)].insert({std::get<1>(m.first), std::get<2>(m.first)});
    return r;
  }

  // A thread evaluates cells c0 .. c0 + V - 1 of a row; V = 4 makes its
  // loads of 4- and 8-byte arrays row vectors (below).
  void cells_per_thread(int V) { V_ = V; }

  // whether the V cells of a row of this type move as one vector
  static bool vector_type(Type t) { return t == TInt || t == TFloat || t == TDouble; }

 private:
  static std::string off_name(int o) { return o < 0 ? "m" + std::to_string(-o) : std::to_string(o); }

  // The element at column c0 + o0 of row c1 + o1 of a global array.  With
  // four cells per thread, the thread's own four columns of a row come in
  // one aligned vector load (rows are whole multiples of 1024 cells, so
  // c0 + 4k is 16-byte aligned for 4-byte types), and the columns of the
  // four before or after come from the neighbouring lane, which loaded
  // them as its own.  Lanes 0 and 31 have no such neighbour in the warp
  // and load that column themselves.  Every lane runs the shuffles (the
  // stage body is straight-line code), and the addresses read are the
  // ones the per-cell loads would read.
  std::string element(const std::string &base, Type t, int o0, int o1) {
    const std::string T = ctype(t);
    const std::string scalar = "((const " + T + " *)" + base + ")[" + addr(o0, o1) + "]";
    if (V_ != 4 || !vector_type(t)) return scalar;
    const int k = o0 >= 0 ? o0 / 4 : -((3 - o0) / 4);  // floor(o0 / 4)
    const int j = o0 - 4 * k;
    if (k < -1 || k > 1) return scalar;
    const std::string own = row_vector(base, t, o1)[j];
    if (k == 0) return own;
    const std::string name = "n" + std::to_string(nshfl_++);
    code += "      const " + T + " " + name + " = " +
            (k < 0 ? "__shfl_up_sync" : "__shfl_down_sync") + "(0xffffffffu, " + own + ", 1);\n";
    return "((threadIdx.x & 31) == " + std::string(k < 0 ? "0" : "31") + " ? " + scalar + " : " +
           name + ")";
  }

  // the four components of the thread's own vector of row c1 + o1
  std::vector<std::string> row_vector(const std::string &base, Type t, int o1) {
    const auto key = std::make_pair(base, o1);
    auto it = vecs_.find(key);
    if (it != vecs_.end()) return it->second;
    const std::string T = ctype(t), y = row(o1);
    const std::string name = "a" + std::to_string(vecs_.size());
    std::vector<std::string> c;
    if (t == TDouble) {
      for (int h = 0; h < 2; ++h)
        code += "      const om_v2d " + name + (h ? "h" : "l") + " = *(const om_v2d *)((const double *)" +
                base + " + " + y + " + c0" + (h ? " + 2" : "") + ");\n";
      c = {name + "l.x", name + "l.y", name + "h.x", name + "h.y"};
    } else {
      const std::string VT = t == TInt ? "om_v4i" : "om_v4f";
      code += "      const " + VT + " " + name + " = *(const " + VT + " *)((const " + T + " *)" + base +
              " + " + y + " + c0);\n";
      c = {name + ".x", name + ".y", name + ".z", name + ".w"};
    }
    return vecs_[key] = c;
  }

  std::string wrap(const std::string &c, int o, int n) const {
    if (o == 0) return c;
    const std::string x = "(" + c + " + (" + std::to_string(o) + "))";
    const std::string N = std::to_string(n);
    if (o > -n && o < n)  // one add or subtract brings it back
      return "(" + x + (o < 0 ? " < 0 ? " + x + " + " + N : " >= " + N + " ? " + x + " - " + N) +
             " : " + x + ")";
    return "((" + x + " % " + N + " + " + N + ") % " + N + ")";
  }

  void select_group(int c, int o0, int o1) {
    const std::string cv = value(c, o0, o1);
    std::vector<int> todo;
    for (int sid : groups_.at(c))
      if (!memo_.count(std::make_tuple(sid, o0, o1))) todo.push_back(sid);
    std::vector<std::string> names;
    for (int sid : todo) {
      const std::string v = "v" + std::to_string(sid) + "_" + off_name(o0) + "_" + off_name(o1);
      code += "      " + std::string(ctype(k_.node(sid).type)) + " " + v + ";\n";
      names.push_back(v);
    }
    open_.insert(std::make_tuple(c, o0, o1));
    const auto memo0 = memo_;
    const auto cols0 = cols_;
    const auto rows0 = rows_;
    for (int side = 1; side <= 2; ++side) {
      code += side == 1 ? "      if (" + cv + ") {\n" : "      } else {\n";
      for (size_t i = 0; i < todo.size(); ++i) {
        const std::string x = value(k_.node(todo[i]).args[side], o0, o1);
        code += "      " + names[i] + " = " + x + ";\n";
      }
      memo_ = memo0;
      cols_ = cols0;
      rows_ = rows0;
    }
    code += "      }\n";
    open_.erase(std::make_tuple(c, o0, o1));
    for (size_t i = 0; i < todo.size(); ++i) memo_[std::make_tuple(todo[i], o0, o1)] = names[i];
  }

  // the column c0 + o (wrapped on a cyclic mesh) and the memory offset of
  // row c1 + o, each declared once per cell and shared by every load
  std::string col(int o) {
    if (o == 0) return "c0";
    auto it = cols_.find(o);
    if (it != cols_.end()) return it->second;
    const std::string name = "x" + off_name(o);
    const std::string e =
        L_.open ? "(c0 + (" + std::to_string(o) + "))" : wrap("c0", o, L_.ms[0]);
    code += "      const int " + name + " = " + e + ";\n";
    return cols_[o] = name;
  }

  std::string row(int o) {
    auto it = rows_.find(o);
    if (it != rows_.end()) return it->second;
    const std::string name = "y" + off_name(o);
    const std::string r =
        L_.open ? "(c1 + (" + std::to_string(o) + "))" : wrap("c1", o, L_.ms[1]);
    code += "      const long long " + name + " = (long long)" + r + " * " +
            std::to_string(L_.ms[0]) + ";\n";
    return rows_[o] = name;
  }

  std::string addr(int o0, int o1) {
    const std::string y = row(o1);
    return y + " + " + col(o0);
  }

  std::string scalar_read(const StaticDef &s) const {
    const std::string off = std::to_string(s.offset);
    if (s.type == TBool) return "(*(const int *)(SC + " + off + ") != 0)";
    return "(*(const " + std::string(ctype(s.type)) + " *)(SC + " + off + "))";
  }

  std::string arith(const Node &n, const std::vector<std::string> &a) const {
    const std::string &op = n.op;
    const std::string T = ctype(n.type);
    auto bin = [&](const char *o) { return "(" + a[0] + " " + o + " " + a[1] + ")"; };
    if (op == "add") return bin("+");
    if (op == "sub") return bin("-");
    if (op == "mul") return bin("*");
    if (op == "div") return bin("/");
    if (op == "mod") return bin("%");
    if (op == "neg") return "(-" + a[0] + ")";
    if (op == "inv") return "(1 / " + a[0] + ")";
    if (op == "not") return "(!" + a[0] + ")";
    if (op == "and") return bin("&&");
    if (op == "or") return bin("||");
    if (op == "eq") return bin("==");
    if (op == "ne") return bin("!=");
    if (op == "lt") return bin("<");
    if (op == "le") return bin("<=");
    if (op == "gt") return bin(">");
    if (op == "ge") return bin(">=");
    if (op == "select") return "(" + a[0] + " ? " + a[1] + " : " + a[2] + ")";
    // std::max(a, b) = (a < b) ? b : a;  std::min(a, b) = (b < a) ? b : a
    if (op == "max") return "((" + a[0] + " < " + a[1] + ") ? " + a[1] + " : " + a[0] + ")";
    if (op == "min") return "((" + a[1] + " < " + a[0] + ") ? " + a[1] + " : " + a[0] + ")";
    if (op == "abs") return n.type == TInt ? "abs(" + a[0] + ")" : "fabs(" + a[0] + ")";
    if (op == "signum")
      return "((" + T + ")((" + a[0] + " > (" + T + ")0) - (" + a[0] + " < (" + T + ")0)))";
    if (op == "cast") return "((" + T + ")(" + a[0] + "))";
    if (op == "atan2" || op == "pow") return op + "(" + a[0] + ", " + a[1] + ")";
    return op + "(" + a[0] + ")";  // sqrt exp log sin cos tan asin acos atan
  }

  const Graph &g_;
  const KernelDef &k_;
  const Layout &L_;
  const std::map<int, int> &slots_;
  const std::map<int, ManifestAt> *man_;
  int stage_;
  std::map<std::tuple<int, int, int>, std::string> memo_;
  std::map<int, std::string> cols_, rows_;
  std::map<std::pair<std::string, int>, std::vector<std::string>> vecs_;
  int V_ = 1, nshfl_ = 0;
  bool lazy_ = false;
  std::map<int, std::vector<int>> groups_;     // condition -> array selects on it
  std::set<std::tuple<int, int, int>> open_;   // (condition, offset) being emitted
  const std::map<int, TileAt> *tiles_ = nullptr;
  TileShape shape_;
};

static std::string region_test(const Region &r, const Layout &L) {
  if (!L.open) return "true";
  std::string t = "true";
  for (int d = 0; d < 2; ++d) {
    const std::string c = d == 0 ? "c0" : "c1";
    const Iv &a = r.ax[d];
    if (!a.lo_inf) t += " && " + c + " >= " + std::to_string(a.lo);
    if (!a.hi_inf) t += " && " + c + " < " + std::to_string(L.ms[d] + a.hi);
  }
  return t;
}

static bool region_is_all(const Region &r, const Layout &L) {
  if (!L.open) return true;
  for (int d = 0; d < 2; ++d) {
    const Iv &a = r.ax[d];
    if (!a.lo_inf && a.lo > 0) return false;
    if (!a.hi_inf && a.hi < 0) return false;
  }
  return true;
}

struct StagePlan {
  std::vector<int> stores;     // indices into KernelDef::stores (array stores)
  std::vector<int> reduces;    // reduce node ids
  std::vector<int> manifests;  // manifest node ids computed by this stage
  std::string fn;
};

struct KernelPlan {
  std::vector<StagePlan> stages;
  std::vector<std::pair<int, Type>> manifest_types;  // temporary array -> element type
  std::vector<int> scalar_stores;  // indices into KernelDef::stores
  std::vector<int> stored_arrays;  // static indices of arrays written
  std::string commit_fn;
};

static const char *kPrelude =
    "struct OMPtrs { const void *cur[32]; void *nxt[32]; void *tmp[64]; };\n"
    "__device__ __forceinline__ float om_inf_f() { return __int_as_float(0x7f800000); }\n"
    "__device__ __forceinline__ double om_inf_d() {\n"
    "  return __longlong_as_double(0x7ff0000000000000LL); }\n"
    "struct alignas(16) om_v4i { int x, y, z, w; };\n"
    "struct alignas(16) om_v4f { float x, y, z, w; };\n"
    "struct alignas(16) om_v2d { double x, y; };\n";

static std::string ident(Type t, const std::string &op) {
  if (op == "sum") return std::string("(") + ctype(t) + ")0";
  const bool mn = op == "min";
  if (t == TInt) return mn ? "2147483647" : "(-2147483647 - 1)";
  if (t == TFloat) return mn ? "om_inf_f()" : "(-om_inf_f())";
  return mn ? "om_inf_d()" : "(-om_inf_d())";
}

static std::string combine(const std::string &op, const std::string &acc, const std::string &x) {
  if (op == "sum") return acc + " + " + x;
  // std::min(acc, x) = (x < acc) ? x : acc;  std::max(acc, x) = (acc < x) ? x : acc
  if (op == "min") return "((" + x + " < " + acc + ") ? " + x + " : " + acc + ")";
  return "((" + acc + " < " + x + ") ? " + x + " : " + acc + ")";
}

// Builds the plan and the CUDA source of every kernel of the graph.
// The outputs a stage evaluates at offset 0 of each cell: its array stores,
// its reduce inputs and the manifests it computes.
static std::vector<int> stage_roots(const KernelDef &k, const StagePlan &sp) {
  std::vector<int> r;
  for (int s : sp.stores) r.push_back(k.stores[s].node);
  for (int id : sp.reduces) r.push_back(k.node(id).args[0]);
  for (int id : sp.manifests) r.push_back(id);
  return r;
}

// Tiled stages.  Where a stage evaluates a computed value at three or more
// offsets of each cell (Hydro's stage-1 state, which each stage-2 wall
// reads at four cells along its axis), recomputing it per offset costs more
// than computing it once per cell of a shared-memory tile.  A tiled stage
// runs in two phases per 32 x 8 tile of cells:
//   1. every value of the frontier (below) for each cell of the tile and its
//      halo, into shared memory;
//   2. the stage's outputs for the tile's cells, reading frontier values
//      from shared memory at their offsets.
// The frontier is the set of values evaluated at three or more offsets that
// an output is, or that a value evaluated at fewer offsets uses; values
// below it are computed in phase 1 only.  The arithmetic of each value is
// unchanged, so results are the same bit for bit (the per-thread order of a
// reduce's terms changes, as with any change of work split).  Cyclic 2-D
// meshes only, whose wrapped neighbours are translation invariant: the value
// at offset o of cell c is the value at offset 0 of cell c + o.
constexpr int kTileSmemBytes = 40 * 1024;

static bool plan_tiles(const Graph &g, const KernelDef &k, const Layout &L,
                       const std::map<int, int> &slots, const std::map<int, ManifestAt> &man,
                       int st, const StagePlan &sp, std::map<int, TileAt> *tiles,
                       TileShape *shape) {
  const std::vector<int> roots = stage_roots(k, sp);
  Emitter trial(g, k, L, slots, &man, st);
  for (int r : roots) trial.value(r, 0, 0);
  const auto offs = trial.offsets();
  auto computed = [&](int id) {
    const Node &n = k.node(id);
    if (!n.array) return false;
    static const std::set<std::string> leaf = {"load",     "imm",    "shift",    "loadindex",
                                               "loadsize", "reduce", "broadcast"};
    if (leaf.count(n.op)) return false;
    auto mi = man.find(id);
    return !(mi != man.end() && mi->second.stage < st);  // else read from its array
  };
  std::set<int> many;
  for (const auto &o : offs)
    if (o.second.size() >= 3 && computed(o.first)) many.insert(o.first);
  if (many.empty()) return false;
  std::set<int> front;
  for (int r : roots)
    if (many.count(r)) front.insert(r);
  for (const auto &o : offs) {
    if (many.count(o.first)) continue;
    for (int a : k.node(o.first).args)
      if (many.count(a)) front.insert(a);
  }
  // keep what phase 2 reads; the halo covers the offsets it reads them at
  for (int round = 0; round < 2; ++round) {
    tiles->clear();
    for (int id : front) (*tiles)[id] = TileAt{"tile" + std::to_string(id)};
    Emitter second(g, k, L, slots, &man, st);
    second.tiled(tiles, TileShape());
    for (int r : roots) second.value(r, 0, 0);
    const auto used = second.offsets();
    std::set<int> kept;
    TileShape sh;
    for (int id : front) {
      auto u = used.find(id);
      if (u == used.end()) continue;
      kept.insert(id);
      for (const auto &o : u->second) {
        sh.hx0 = std::max(sh.hx0, -o.first);
        sh.hx1 = std::max(sh.hx1, o.first);
        sh.hy0 = std::max(sh.hy0, -o.second);
        sh.hy1 = std::max(sh.hy1, o.second);
      }
    }
    *shape = sh;
    if (kept == front) break;
    front = kept;
  }
  if (front.empty()) return false;
  tiles->clear();
  size_t bytes = 0;
  double reads = 0;
  for (int id : front) {
    (*tiles)[id] = TileAt{"tile" + std::to_string(id)};
    bytes += (size_t)shape->rx() * shape->ry() * tsize(k.node(id).type);
    reads += offs.at(id).size();
  }
  const double cells = (double)shape->rx() * shape->ry() / (shape->tx * shape->ty);
  if (bytes > (size_t)kTileSmemBytes || shape->hx0 > 8 || shape->hx1 > 8 || shape->hy0 > 8 ||
      shape->hy1 > 8)
    return false;
  // worth it when the frontier values were evaluated at clearly more
  // offsets per cell than the tile computes them
  return reads / front.size() >= 1.5 * cells;
}

static void emit_tiled(std::ostringstream &src, const Graph &g, const KernelDef &k,
                       const Layout &L, const std::map<int, int> &slots,
                       const std::map<int, ManifestAt> &man, int st, const StagePlan &sp,
                       const std::map<int, TileAt> &tiles, const TileShape &sh,
                       Emitter &names) {
  const int RX = sh.rx(), RY = sh.ry();
  const std::string n0 = std::to_string(L.ms[0]), n1 = std::to_string(L.ms[1]);
  for (const auto &t : tiles)
    src << "  __shared__ " << ctype(k.node(t.first).type) << " " << t.second.name << "["
        << RX * RY << "];\n";
  src << "  constexpr int NTX = " << (L.ms[0] + sh.tx - 1) / sh.tx
      << ", NTY = " << (L.ms[1] + sh.ty - 1) / sh.ty << ";\n"
      << "  for (long long w = blockIdx.x; w < (long long)NTX * NTY; w += gridDim.x) {\n"
      << "    const int X0 = (int)(w % NTX) * " << sh.tx << ", Y0 = (int)(w / NTX) * " << sh.ty
      << ";\n"
      << "    __syncthreads();  // the previous tile's phase 2 is done with the tiles\n"
      << "    for (int e = threadIdx.x; e < " << RX * RY << "; e += 256) {\n"
      << "      const int ry = e / " << RX << ", rx = e - ry * " << RX << ";\n"
      << "      const int c0 = ((X0 + rx - " << sh.hx0 << ") % " << n0 << " + " << n0 << ") % "
      << n0 << ";\n"
      << "      const int c1 = ((Y0 + ry - " << sh.hy0 << ") % " << n1 << " + " << n1 << ") % "
      << n1 << ";\n"
      << "      const long long i = (long long)c1 * " << n0 << " + c0;\n"
      << "      (void)i;\n";
  {
    Emitter first(g, k, L, slots, &man, st);
    first.lazy_selects(true);
    std::vector<std::string> vals;
    for (const auto &t : tiles) vals.push_back(first.value(t.first, 0, 0));
    src << "    {\n" << first.code;
    size_t v = 0;
    for (const auto &t : tiles) src << "      " << t.second.name << "[e] = " << vals[v++] << ";\n";
    src << "    }\n";
  }
  src << "    }\n    __syncthreads();\n"
      << "    for (int e = threadIdx.x; e < " << sh.tx * sh.ty << "; e += 256) {\n"
      << "      const int ty = e / " << sh.tx << ", tx = e - ty * " << sh.tx << ";\n"
      << "      const int c0 = X0 + tx, c1 = Y0 + ty;\n"
      << "      if (c0 >= " << n0 << " || c1 >= " << n1 << ") continue;\n"
      << "      const long long i = (long long)c1 * " << n0 << " + c0;\n";
  Emitter second(g, k, L, slots, &man, st);
  second.lazy_selects(true);
  second.tiled(&tiles, sh);
  std::vector<std::string> vals;
  for (int r : stage_roots(k, sp)) vals.push_back(second.value(r, 0, 0));
  src << "    {\n" << second.code;
  size_t v = 0;
  for (int s : sp.stores)
    src << "      ((" << ctype(k.node(k.stores[s].node).type) << " *)P.nxt["
        << names.array_index(k.stores[s].stat) << "])[i] = " << vals[v++] << ";\n";
  for (size_t r = 0; r < sp.reduces.size(); ++r) {
    const std::string acc = "acc" + std::to_string(r);
    src << "      " << acc << " = " << combine(k.node(sp.reduces[r]).sarg, acc, vals[v++]) << ";\n";
  }
  for (int id : sp.manifests)
    src << "      ((" << ctype(k.node(id).type) << " *)P.tmp[" << man.at(id).tmp << "])[i] = "
        << vals[v++] << ";\n";
  src << "    }\n    }\n  }\n";
}

static std::string generate(const Graph &g, const Layout &L, std::vector<KernelPlan> *plans,
                            std::map<std::pair<int, int>, int> *slot_map, int *nslots,
                            int *ntmp) {
  std::ostringstream src;
  src << kPrelude;
  int slot = 0;
  *ntmp = 0;
  for (size_t ki = 0; ki < g.kernels.size(); ++ki) {
    const KernelDef &k = g.kernels[ki];
    KernelPlan kp;
    const std::vector<Region> reg = regions(k);
    // the last store to each static wins (manifests are copied in order)
    std::vector<int> last(g.statics.size(), -1);
    for (size_t s = 0; s < k.stores.size(); ++s) last[k.stores[s].stat] = (int)s;
    // manifests in use: reachable from a store that counts or a reduce
    std::set<int> live;
    {
      std::vector<int> todo;
      for (size_t s = 0; s < k.stores.size(); ++s)
        if (last[k.stores[s].stat] == (int)s) todo.push_back(k.stores[s].node);
      for (const Node &n : k.nodes)
        if (n.op == "reduce") todo.push_back(n.id);
      while (!todo.empty()) {
        const int id = todo.back();
        todo.pop_back();
        if (!live.insert(id).second) continue;
        for (int a : k.node(id).args) todo.push_back(a);
      }
    }
    // the stage (kernel pass) in which each value is first available: a
    // reduce's or a manifest's value only in the pass after the one that
    // computes it; other values wherever their operands are
    std::vector<int> avail(k.nodes.size(), 0);
    std::map<int, int> slots;
    std::map<int, ManifestAt> man;
    for (size_t i = 0; i < k.nodes.size(); ++i) {
      const Node &n = k.nodes[i];
      int d = 0;
      for (int a : n.args) d = std::max(d, avail[k.at.at(a)]);
      if (n.op == "reduce") {
        slots[n.id] = slot;
        (*slot_map)[{(int)ki, n.id}] = slot++;
        d += 1;
      } else if (k.manifest.count(n.id) && live.count(n.id)) {
        man[n.id] = ManifestAt{d, (*ntmp)++};
        d += 1;
      }
      avail[i] = d;
    }
    // the pass that computes a value a store, a reduce or a manifest needs
    auto comp = [&](int id) {
      auto mi = man.find(id);
      return mi != man.end() ? mi->second.stage : avail[k.at.at(id)];
    };
    int nst = 0;
    for (size_t s = 0; s < k.stores.size(); ++s) {
      if (last[k.stores[s].stat] != (int)s) continue;
      const int id = k.stores[s].node;
      if (g.statics[k.stores[s].stat].array) {
        nst = std::max(nst, comp(id) + 1);
        kp.stored_arrays.push_back(k.stores[s].stat);
      } else {
        kp.scalar_stores.push_back((int)s);
      }
    }
    for (const Node &n : k.nodes)
      if (n.op == "reduce") nst = std::max(nst, comp(n.args[0]) + 1);
    for (const auto &m : man) nst = std::max(nst, m.second.stage + 1);
    kp.stages.resize(nst);
    for (size_t s = 0; s < k.stores.size(); ++s)
      if (last[k.stores[s].stat] == (int)s && g.statics[k.stores[s].stat].array)
        kp.stages[comp(k.stores[s].node)].stores.push_back((int)s);
    for (const Node &n : k.nodes)
      if (n.op == "reduce") kp.stages[comp(n.args[0])].reduces.push_back(n.id);
    for (const auto &m : man) {
      kp.stages[m.second.stage].manifests.push_back(m.first);
      kp.manifest_types.push_back({m.second.tmp, k.node(m.first).type});
    }

    for (int st = 0; st < nst; ++st) {
      StagePlan &sp = kp.stages[st];
      sp.fn = "om_k" + std::to_string(ki) + "_s" + std::to_string(st);
      Emitter em(g, k, L, slots, &man, st);
      std::ostringstream body;
      src << "extern \"C\" __global__ void __launch_bounds__(256)\n" << sp.fn
          << "(OMPtrs P, const unsigned char *SC, unsigned char *slots, unsigned char *part,\n"
          << "     unsigned int *done) {\n";
      for (size_t r = 0; r < sp.reduces.size(); ++r) {
        const Node &n = k.node(sp.reduces[r]);
        src << "  " << ctype(n.type) << " acc" << r << " = " << ident(n.type, n.sarg) << ";\n";
      }
      // one evaluation block for the whole stage when every store and reduce
      // of it has the same region (always so on a cyclic mesh): the values
      // they share are computed once per cell
      std::vector<std::string> tests;
      for (int s : sp.stores) tests.push_back(region_test(reg[k.at.at(k.stores[s].node)], L));
      for (int id : sp.reduces) tests.push_back(region_test(reg[k.at.at(k.node(id).args[0])], L));
      for (int id : sp.manifests) tests.push_back(region_test(reg[k.at.at(id)], L));
      bool one_region = !tests.empty();
      for (const std::string &t : tests) one_region = one_region && t == tests[0];
      bool all_cells = true;
      for (int id : sp.reduces) all_cells = all_cells && region_is_all(reg[k.at.at(k.node(id).args[0])], L);
      const bool shared = one_region && all_cells && tests[0] == "true";
      // cells per thread: a thread evaluates V neighbouring cells of a row as
      // offsets 0 .. V-1 of its first one, so loads they share are made once
      // and V cells' loads are in flight together (small stages on rows that
      // are whole multiples of 256 V cells)
      int V = 1;
      if (shared && L.ms[0] % (256 * kCellsPerThread) == 0) {
        Emitter trial(g, k, L, slots, &man, st);
        for (int s : sp.stores) trial.value(k.stores[s].node, 0, 0);
        for (int id : sp.reduces) trial.value(k.node(id).args[0], 0, 0);
        for (int id : sp.manifests) trial.value(id, 0, 0);
        // a stage that selects whole records (two or more selects on one
        // condition) stays at one cell per thread, where it can branch on
        // the condition instead (Emitter::lazy_selects)
        std::map<int, int> on_condition;
        for (const auto &o : trial.offsets()) {
          const Node &n = k.node(o.first);
          if (n.op == "select" && n.array) ++on_condition[n.args[0]];
        }
        bool records = false;
        for (const auto &c : on_condition) records = records || c.second >= 2;
        if (!records &&
            std::count(trial.code.begin(), trial.code.end(), '\n') <= kMaxVectorStatements)
          V = kCellsPerThread;
      }
      std::map<int, TileAt> tiles;
      TileShape shape;
      const bool tiled = V == 1 && shared && !L.open && g.ndim == 2 &&
                         plan_tiles(g, k, L, slots, man, st, sp, &tiles, &shape);
      if (tiled) {
        emit_tiled(src, g, k, L, slots, man, st, sp, tiles, shape, em);
      } else {
        // work items: chunks of 256 V cells of a memory row, rows in order; a
        // block takes items blockIdx.x, blockIdx.x + gridDim.x, ...
        const int chunk = 256 * V;
        src << "  constexpr int CX = " << (L.ms[0] + chunk - 1) / chunk << ";\n"
            << "  const long long NW = (long long)" << L.ms[1] << " * CX;\n"
            << "  for (long long w = blockIdx.x; w < NW; w += gridDim.x) {\n"
            << "    const int c1 = (int)(w / CX);\n"
            << "    const int c0 = (int)(w - (long long)c1 * CX) * " << chunk << " + (int)threadIdx.x";
        if (V > 1) src << " * " << V;
        src << ";\n";
        if (V == 1) src << "    if (c0 >= " << L.ms[0] << ") continue;\n";
        src << "    const long long i = (long long)c1 * " << L.ms[0] << " + c0;\n"
            << "    (void)c0; (void)c1;\n";
        if (shared) {
          Emitter e(g, k, L, slots, &man, st);
          e.cells_per_thread(V);
          e.lazy_selects(V == 1);
          // vals[c][...]: cell c's stores, reduce inputs and manifests
          std::vector<std::vector<std::string>> vals(V);
          for (int c = 0; c < V; ++c) {
            for (int s : sp.stores) vals[c].push_back(e.value(k.stores[s].node, c, 0));
            for (int id : sp.reduces) vals[c].push_back(e.value(k.node(id).args[0], c, 0));
            for (int id : sp.manifests) vals[c].push_back(e.value(id, c, 0));
          }
          src << "    {\n" << e.code;
          // the V cells' values of one array go out as one store (a vector
          // of 4 for 4- and 8-byte types, at 16-byte aligned i)
          auto store = [&](Type t, const std::string &ptr, size_t slot) {
            const std::string T = ctype(t);
            if (V == 4 && Emitter::vector_type(t)) {
              const std::string p = "((" + T + " *)" + ptr + " + i";
              if (t == TDouble)
                src << "      *(om_v2d *)" << p << ") = om_v2d{" << vals[0][slot] << ", "
                    << vals[1][slot] << "};\n      *(om_v2d *)" << p << " + 2) = om_v2d{"
                    << vals[2][slot] << ", " << vals[3][slot] << "};\n";
              else
                src << "      *(" << (t == TInt ? "om_v4i" : "om_v4f") << " *)" << p << ") = "
                    << (t == TInt ? "om_v4i{" : "om_v4f{") << vals[0][slot] << ", " << vals[1][slot]
                    << ", " << vals[2][slot] << ", " << vals[3][slot] << "};\n";
              return;
            }
            for (int c = 0; c < V; ++c)
              src << "      ((" << T << " *)" << ptr << ")[" << (c == 0 ? "i" : "i + " + std::to_string(c))
                  << "] = " << vals[c][slot] << ";\n";
          };
          size_t slot0 = 0;
          for (int s : sp.stores)
            store(k.node(k.stores[s].node).type, "P.nxt[" + std::to_string(em.array_index(k.stores[s].stat)) + "]",
                  slot0++);
          // reduces fold the cells in order c = 0 .. V - 1
          for (int c = 0; c < V; ++c)
            for (size_t r = 0; r < sp.reduces.size(); ++r) {
              const std::string acc = "acc" + std::to_string(r);
              src << "      " << acc << " = "
                  << combine(k.node(sp.reduces[r]).sarg, acc, vals[c][sp.stores.size() + r]) << ";\n";
            }
          slot0 += sp.reduces.size();
          for (int id : sp.manifests)
            store(k.node(id).type, "P.tmp[" + std::to_string(man.at(id).tmp) + "]", slot0++);
          src << "    }\n";
        } else {
          // a manifest is written on its region (other cells are never read)
          for (int id : sp.manifests) {
            const std::string T = ctype(k.node(id).type);
            Emitter e(g, k, L, slots, &man, st);
            e.lazy_selects(true);
            const std::string val = e.value(id, 0, 0);
            src << "    {\n      if (" << region_test(reg[k.at.at(id)], L) << ") {\n" << e.code
                << "      ((" << T << " *)P.tmp[" << man.at(id).tmp << "])[i] = " << val << ";\n"
                << "      }\n    }\n";
          }
          for (int s : sp.stores) {
            const Store &so = k.stores[s];
            const Node &v = k.node(so.node);
            const std::string T = ctype(v.type);
            Emitter e(g, k, L, slots, &man, st);
            e.lazy_selects(true);
            const std::string val = e.value(so.node, 0, 0);
            src << "    {\n      " << T << " out = (" << T << ")0;\n"
                << "      if (" << region_test(reg[k.at.at(so.node)], L) << ") {\n"
                << e.code << "      out = " << val << ";\n      }\n"
                << "      ((" << T << " *)P.nxt[" << em.array_index(so.stat) << "])[i] = out;\n"
                << "    }\n";
          }
          for (size_t r = 0; r < sp.reduces.size(); ++r) {
            const Node &n = k.node(sp.reduces[r]);
            const int in = n.args[0];
            Emitter e(g, k, L, slots, &man, st);
            e.lazy_selects(true);
            const std::string val = e.value(in, 0, 0);
            const std::string acc = "acc" + std::to_string(r);
            src << "    {\n      if (" << region_test(reg[k.at.at(in)], L) << ") {\n" << e.code
                << "      " << acc << " = " << combine(n.sarg, acc, val) << ";\n      }";
            if (!region_is_all(reg[k.at.at(in)], L))
              src << " else {\n      " << acc << " = "
                  << combine(n.sarg, acc, std::string("(") + ctype(n.type) + ")0") << ";\n      }";
            src << "\n    }\n";
          }
        }
        src << "  }\n";
      }
      if (!sp.reduces.empty()) {
        // per-block fixed tree, partials, then the last block in block order
        for (size_t r = 0; r < sp.reduces.size(); ++r) {
          const Node &n = k.node(sp.reduces[r]);
          const std::string T = ctype(n.type), acc = "acc" + std::to_string(r);
          const std::string sh = "sh" + std::to_string(r);
          src << "  {\n    __shared__ " << T << " " << sh << "[256];\n"
              << "    " << sh << "[threadIdx.x] = " << acc << ";\n    __syncthreads();\n"
              << "    for (int w = 128; w > 0; w >>= 1) {\n"
              << "      if ((int)threadIdx.x < w) " << sh << "[threadIdx.x] = "
              << combine(n.sarg, sh + "[threadIdx.x]", sh + "[threadIdx.x + w]") << ";\n"
              << "      __syncthreads();\n    }\n"
              << "    if (threadIdx.x == 0) ((" << T << " *)(part + " << r
              << " * 8 * gridDim.x))[blockIdx.x] = " << sh << "[0];\n  }\n";
        }
        src << "  __shared__ bool last;\n  __threadfence();\n  __syncthreads();\n"
            << "  if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;\n"
            << "  __syncthreads();\n"
            << "  if (!last || threadIdx.x != 0) return;\n  __threadfence();\n";
        for (size_t r = 0; r < sp.reduces.size(); ++r) {
          const Node &n = k.node(sp.reduces[r]);
          const std::string T = ctype(n.type);
          src << "  {\n    const volatile " << T << " *p = (const volatile " << T
              << " *)(part + " << r << " * 8 * gridDim.x);\n"
              << "    " << T << " a = p[0];\n"
              << "    for (unsigned int b = 1; b < gridDim.x; ++b) a = "
              << combine(n.sarg, "a", "p[b]") << ";\n"
              << "    *(" << T << " *)(slots + " << 8 * slots.at(sp.reduces[r]) << ") = a;\n"
              << "  }\n";
        }
        src << "  *done = 0;\n";
      }
      src << "}\n\n";
    }
    // scalar stores: one thread evaluates every stored value, then writes
    kp.commit_fn = "om_k" + std::to_string(ki) + "_commit";
    {
      src << "extern \"C\" __global__ void " << kp.commit_fn
          << "(OMPtrs P, unsigned char *SC, unsigned char *slots) {\n"
          << "  if (threadIdx.x != 0 || blockIdx.x != 0) return;\n"
          << "  const int c0 = 0, c1 = 0; (void)c0; (void)c1; (void)P;\n";
      Emitter e(g, k, L, slots);
      std::vector<std::string> vals;
      for (int s : kp.scalar_stores) vals.push_back(e.value(k.stores[s].node, 0, 0));
      src << e.code;
      for (size_t i = 0; i < kp.scalar_stores.size(); ++i) {
        const StaticDef &sd = g.statics[k.stores[kp.scalar_stores[i]].stat];
        if (sd.type == TBool)
          src << "  *(int *)(SC + " << sd.offset << ") = " << vals[i] << " ? 1 : 0;\n";
        else
          src << "  *(" << ctype(sd.type) << " *)(SC + " << sd.offset << ") = " << vals[i]
              << ";\n";
      }
      src << "}\n\n";
    }
    plans->push_back(kp);
  }
  *nslots = slot;
  return src.str();
}

// ---------------------------------------------------------------------------
// the handle kind
// ---------------------------------------------------------------------------

// at most this many manifest values in use across a graph's kernels
constexpr int kMaxManifests = 64;

struct GraphState {
  Graph g;
  Layout L;
  std::vector<KernelPlan> plans;
  std::vector<Type> tmp_types;   // element type of each manifest array
  std::vector<void *> tmp;       // the manifest arrays (memory-sized)
  cudaLibrary_t lib = nullptr;
  std::vector<std::vector<cudaKernel_t>> stage_k;
  std::vector<cudaKernel_t> commit_k;
  unsigned char *slots = nullptr;  // 8 bytes per reduce
  unsigned char *part = nullptr;   // per reduce of a stage: 8 bytes per block
  unsigned int *done = nullptr;    // one counter per (kernel, stage)
  std::vector<std::vector<int>> done_index;
  int grid = 1;
  std::string source;
  bool owned = false;  // freed with the handle once setup has started
};

static GraphState *gst(Handle *h) { return (GraphState *)h->impl; }

static void graph_free(Handle *h) {
  GraphState *st = gst(h);
  if (!st) return;
  if (st->lib) cudaLibraryUnload(st->lib);
  for (void *p : st->tmp) cudaFree(p);
  cudaFree(st->slots);
  cudaFree(st->part);
  cudaFree(st->done);
  delete st;
  h->impl = nullptr;
}

struct OMPtrs {
  const void *cur[32];
  void *nxt[32];
  void *tmp[kMaxManifests];
};

static om_status graph_run(Handle *h, int n) {
  GraphState *st = gst(h);
  const int ki = h->current_kernel;
  const KernelPlan &kp = st->plans[ki];
  for (int rep = 0; rep < n; ++rep) {
    OMPtrs P;
    std::memset(&P, 0, sizeof P);
    for (size_t a = 0; a < h->arrays.size(); ++a) {
      P.cur[a] = h->arrays[a].d();
      P.nxt[a] = h->arrays[a].d_next();
    }
    for (size_t t = 0; t < st->tmp.size(); ++t) P.tmp[t] = st->tmp[t];
    unsigned char *SC = (unsigned char *)h->d_scalars;
    for (size_t s = 0; s < kp.stages.size(); ++s) {
      unsigned int *done = st->done + st->done_index[ki][s];
      void *args[] = {&P, &SC, &st->slots, &st->part, &done};
      OM_CUDA_CHECK(cudaLaunchKernel((const void *)st->stage_k[ki][s], dim3(st->grid), dim3(256),
                                     args, 0, h->stream));
      h->launches++;
    }
    if (!kp.scalar_stores.empty()) {
      void *args[] = {&P, &SC, &st->slots};
      OM_CUDA_CHECK(cudaLaunchKernel((const void *)st->commit_k[ki], dim3(1), dim3(32), args, 0,
                                     h->stream));
      h->launches++;
    }
    for (int s : kp.stored_arrays) {
      int a = 0;
      for (int i = 0; i < s; ++i) a += st->g.statics[i].array ? 1 : 0;
      h->arrays[a].swap();
    }
  }
  return OM_OK;
}

// NVRTC: the generated source to a cubin for sm_<major><minor>a
static om_status nvrtc_cubin(const std::string &source, int major, int minor,
                             std::vector<char> *cubin) {
  nvrtcProgram prog;
  if (nvrtcCreateProgram(&prog, source.c_str(), "omgraph.cu", 0, nullptr, nullptr) !=
      NVRTC_SUCCESS) {
    set_error("om_create_graph: nvrtcCreateProgram failed");
    return OM_ERR_CUDA;
  }
  const std::string arch =
      "--gpu-architecture=sm_" + std::to_string(major) + std::to_string(minor) + "a";
  const char *opts[] = {arch.c_str(), "--fmad=false", "--std=c++17"};
  const nvrtcResult r = nvrtcCompileProgram(prog, 3, opts);
  if (r != NVRTC_SUCCESS) {
    size_t n = 0;
    nvrtcGetProgramLogSize(prog, &n);
    std::string log(n, '\0');
    nvrtcGetProgramLog(prog, &log[0]);
    nvrtcDestroyProgram(&prog);
    set_error("om_create_graph: NVRTC: " + std::string(nvrtcGetErrorString(r)) + "\n" + log);
    return OM_ERR_CUDA;
  }
  size_t bytes = 0;
  nvrtcGetCUBINSize(prog, &bytes);
  cubin->resize(bytes);
  nvrtcGetCUBIN(prog, cubin->data());
  nvrtcDestroyProgram(&prog);
  return OM_OK;
}

static om_status compile(GraphState *st, int device) {
  int major = 0, minor = 0;
  OM_CUDA_CHECK(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device));
  OM_CUDA_CHECK(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device));
  std::vector<char> cubin;
  OM_TRY(nvrtc_cubin(st->source, major, minor, &cubin));
  OM_CUDA_CHECK(cudaLibraryLoadData(&st->lib, cubin.data(), nullptr, nullptr, 0, nullptr,
                                    nullptr, 0));
  st->stage_k.resize(st->plans.size());
  st->commit_k.resize(st->plans.size());
  for (size_t k = 0; k < st->plans.size(); ++k) {
    for (const StagePlan &sp : st->plans[k].stages) {
      cudaKernel_t f;
      OM_CUDA_CHECK(cudaLibraryGetKernel(&f, st->lib, sp.fn.c_str()));
      st->stage_k[k].push_back(f);
    }
    OM_CUDA_CHECK(cudaLibraryGetKernel(&st->commit_k[k], st->lib, st->plans[k].commit_fn.c_str()));
  }
  return OM_OK;
}

// Margins (the intersection of every array store's region on open axes),
// the memory layout, scalar offsets, the plans and the CUDA source: all
// host-side, no device needed.
static om_status plan(GraphState *st, int *nslots) {
  Graph &g = st->g;
  Layout &L = st->L;
  L.open = g.open;
  Region united;
  for (const KernelDef &k : g.kernels) {
    const std::vector<Region> reg = regions(k);
    for (const Store &s : k.stores)
      if (g.statics[s.stat].array) united = meet(united, reg[k.at.at(s.node)]);
  }
  for (int d = 0; d < 2; ++d) {
    const bool axis_open = g.open && d < g.ndim;
    const int lo = (!axis_open || united.ax[d].lo_inf) ? 0 : united.ax[d].lo;
    const int hi = (!axis_open || united.ax[d].hi_inf) ? 0 : -united.ax[d].hi;
    if (lo < 0 || hi < 0) {
      set_error("om_create_graph: negative margin (a store reaches beyond the array)");
      return OM_ERR_ARG;
    }
    L.lm[d] = lo;
    L.size[d] = g.size[d];
    L.ms[d] = g.size[d] + lo + hi;
  }
  int narrays = 0;
  size_t off = 0;
  for (StaticDef &s : g.statics) {
    if (s.array) {
      if (++narrays > 32) {
        set_error("om_create_graph: at most 32 array statics");
        return OM_ERR_UNSUPPORTED;
      }
    } else {
      s.offset = off;
      off += 8;
    }
  }
  std::map<std::pair<int, int>, int> slot_map;
  st->plans.clear();
  int ntmp = 0;
  st->source = generate(g, L, &st->plans, &slot_map, nslots, &ntmp);
  if (ntmp > kMaxManifests) {
    set_error("om_create_graph: at most " + std::to_string(kMaxManifests) +
              " manifest values in use");
    return OM_ERR_UNSUPPORTED;
  }
  st->tmp_types.assign(ntmp, TInt);
  for (const KernelPlan &kp : st->plans)
    for (const auto &m : kp.manifest_types) st->tmp_types[m.first] = m.second;
  return OM_OK;
}

static om_status graph_setup(Handle *h, void *ctx) {
  GraphState *st = (GraphState *)ctx;
  st->owned = true;
  h->impl = st;
  h->impl_free = graph_free;
  Graph &g = st->g;
  const Layout &L = st->L;
  int nslots = 0;
  OM_TRY(plan(st, &nslots));
  for (int d = 0; d < 2; ++d) {
    h->lower_margin[d] = L.lm[d];
    h->upper_margin[d] = L.ms[d] - L.size[d] - L.lm[d];
  }
  size_t scalar_end = 8;
  for (StaticDef &s : g.statics) {
    if (s.array) {
      OM_TRY(alloc_array(h, s.name.c_str(), tsize(s.type)));
    } else {
      h->scalars.push_back(
          {s.name, s.type == TDouble ? kDouble : (s.type == TFloat ? kFloat : kInt), s.offset});
      scalar_end = std::max(scalar_end, s.offset + 8);
    }
  }
  h->scalar_bytes = scalar_end;
  for (const KernelDef &k : g.kernels) h->kernels.push_back({k.name, graph_run});
  const long long cells = (long long)L.ms[0] * L.ms[1];
  st->grid = (int)std::max<long long>(
      1, std::min<long long>((cells + 255) / 256, 8LL * sm_count(h->device)));
  int maxred = 1, nstages = 0;
  st->done_index.resize(st->plans.size());
  for (size_t k = 0; k < st->plans.size(); ++k)
    for (const StagePlan &sp : st->plans[k].stages) {
      maxred = std::max(maxred, (int)sp.reduces.size());
      st->done_index[k].push_back(nstages++);
    }
  for (Type t : st->tmp_types) {
    void *p = nullptr;
    if (injected_alloc_failure() ||
        cudaMalloc(&p, (size_t)tsize(t) * h->memory_size_total()) != cudaSuccess) {
      cudaGetLastError();
      set_error("om_create_graph: cannot allocate the manifest arrays");
      return OM_ERR_NOMEM;
    }
    st->tmp.push_back(p);
  }
  if (cudaMalloc(&st->slots, 8 * (size_t)std::max(nslots, 1)) != cudaSuccess ||
      cudaMalloc(&st->part, 8 * (size_t)maxred * st->grid) != cudaSuccess ||
      cudaMalloc(&st->done, sizeof(unsigned int) * std::max(nstages, 1)) != cudaSuccess ||
      cudaMemset(st->done, 0, sizeof(unsigned int) * std::max(nstages, 1)) != cudaSuccess ||
      cudaMemset(st->slots, 0, 8 * (size_t)std::max(nslots, 1)) != cudaSuccess) {
    cudaGetLastError();
    set_error("om_create_graph: allocation failed");
    return OM_ERR_NOMEM;
  }
  return compile(st, h->device);
}

}  // namespace og
}  // namespace om

using namespace om;

extern "C" om_status om_create_graph(const char *text, const om_config *cfg, om_handle *out) {
  if (!text || !out) {
    set_error("om_create_graph: null argument");
    return OM_ERR_ARG;
  }
  *out = nullptr;
  og::GraphState *st = new og::GraphState();
  om_status s = og::parse(text, &st->g);
  if (s != OM_OK) {
    delete st;
    return s;
  }
  om_config c;
  if (cfg) c = *cfg; else om_config_default(&c);
  c.boundary = st->g.open ? OM_BOUNDARY_OPEN : OM_BOUNDARY_CYCLIC;
  const int sizes[2] = {st->g.size[0], st->g.size[1]};
  struct Setup {
    static om_status run(Handle *h, void *ctx) { return og::graph_setup(h, ctx); }
  };
  s = create_handle(OM_KIND_GRAPH, sizes, c, Setup::run, st, out);
  // once setup has run, the handle owns st (and destroyed it on failure)
  if (s != OM_OK && !st->owned) delete st;
  return s;
}

// Parse, plan, generate and compile a graph for sm_<major><minor>a without a
// device; *source (valid until the next call on this thread) receives the
// generated CUDA source.
extern "C" om_status om_graph_check(const char *text, int major, int minor,
                                    const char **source) {
  static thread_local std::string keep;
  if (!text) {
    set_error("om_graph_check: null graph");
    return OM_ERR_ARG;
  }
  og::GraphState st;
  OM_TRY(og::parse(text, &st.g));
  int nslots = 0;
  OM_TRY(og::plan(&st, &nslots));
  keep = st.source;
  if (source) *source = keep.c_str();
  std::vector<char> cubin;
  return og::nvrtc_cubin(st.source, major, minor, &cubin);
}

extern "C" om_status om_graph_source(om_handle H, const char **source) {
  Handle *h = handle_of(H);
  if (!h || h->kind != OM_KIND_GRAPH || !source) {
    set_error("om_graph_source: needs a graph handle");
    return OM_ERR_ARG;
  }
  *source = og::gst(h)->source.c_str();
  return OM_OK;
}
