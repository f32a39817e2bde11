// Per-class program builder for the warp-cooperative ERI kernel (see
// lgx_program.h for the op encoding and the reference anchors).
#include "lgx_program.h"

#include <algorithm>
#include <array>
#include <functional>
#include <map>
#include <stdexcept>
#include <string>
#include <unordered_map>

namespace lgx {
namespace {

constexpr int kCompL = 12;  // component table covers shells 0..kCompL

inline int ncart(int l) { return (l + 1) * (l + 2) / 2; }
inline int cum(int l) { return l * (l + 1) * (l + 2) / 6; }
inline int cart_index(int l, int lx, int ly) {
  const int i = l - lx;
  return i * (i + 1) / 2 + (i - ly);
}
struct C3 {
  int x, y, z;
  int l() const { return x + y + z; }
  int operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline int cidx(const C3& c) { return cum(c.l()) + cart_index(c.l(), c.x, c.y); }
inline C3 shift(C3 c, int i, int d) {
  if (i == 0) c.x += d; else if (i == 1) c.y += d; else c.z += d;
  return c;
}
inline int first_dir(const C3& c) { return c.x ? 0 : (c.y ? 1 : 2); }
std::vector<C3> comps(int l) {
  std::vector<C3> v;
  for (int lx = l; lx >= 0; --lx)
    for (int ly = l - lx; ly >= 0; --ly) v.push_back({lx, ly, l - lx - ly});
  return v;
}

// ------------------------------------------------------------ slot pool
struct SlotPool {
  int base, next = 0, high = 0;
  std::vector<int> free_list;
  explicit SlotPool(int b) : base(b) {}
  int take() {
    if (!free_list.empty()) {
      int s = free_list.back();
      free_list.pop_back();
      return s;
    }
    int s = base + next++;
    high = std::max(high, next);
    return s;
  }
  void give(int s) { free_list.push_back(s); }
};

// ----------------------------------------------------------------- VRR DAG
struct VNode {
  C3 e, f;
  int m;
  int kind = -1;  // -1 leaf, 0 build on A, 1 build on C
  int dir = 0, n1 = 0, ne = 0;
  int src[5] = {-1, -1, -1, -1, -1};
  int level = 0, last_use = -1, slot = -1;
};

struct VrrDag {
  std::vector<VNode> nodes;
  std::unordered_map<int64_t, int> index;
  static int64_t key(const C3& e, const C3& f, int m) {
    return (int64_t(cidx(e)) * 4096 + cidx(f)) * 64 + m;
  }
  int get(const C3& e, const C3& f, int m) {
    const int64_t k = key(e, f, m);
    auto it = index.find(k);
    if (it != index.end()) return it->second;
    VNode n;
    n.e = e;
    n.f = f;
    n.m = m;
    const int id = (int)nodes.size();
    nodes.push_back(n);
    index.emplace(k, id);
    // expand dependencies
    if (f.l() > 0) {
      const int j = first_dir(f);
      const C3 f1 = shift(f, j, -1);
      VNode tmp = nodes[id];
      tmp.kind = 1;
      tmp.dir = j;
      tmp.src[0] = get(e, f1, m);
      tmp.src[1] = get(e, f1, m + 1);
      if (f1[j] > 0) {
        const C3 f2 = shift(f1, j, -1);
        tmp.n1 = f1[j];
        tmp.src[2] = get(e, f2, m);
        tmp.src[3] = get(e, f2, m + 1);
      }
      if (e[j] > 0) {
        tmp.ne = e[j];
        tmp.src[4] = get(shift(e, j, -1), f1, m + 1);
      }
      tmp.e = nodes[id].e;
      nodes[id] = tmp;
    } else if (e.l() > 0) {
      const int i = first_dir(e);
      const C3 e1 = shift(e, i, -1);
      VNode tmp = nodes[id];
      tmp.kind = 0;
      tmp.dir = i;
      tmp.src[0] = get(e1, f, m);
      tmp.src[1] = get(e1, f, m + 1);
      if (e1[i] > 0) {
        const C3 e2 = shift(e1, i, -1);
        tmp.n1 = e1[i];
        tmp.src[2] = get(e2, f, m);
        tmp.src[3] = get(e2, f, m + 1);
      }
      nodes[id] = tmp;
    }
    return id;
  }
};

// --------------------------------------------------------------- post DAG
struct PNode {
  int kind = -1;  // -1: leaf (accumulator slot), else PostKind
  int dir = 0, n = 0;
  int src[3] = {-1, -1, -1};
  int leaf_slot = -1;   // accumulator slot for leaves
  int pinned_slot = -1; // output slot (fixed)
  int level = 0, last_use = -1, slot = -1;
};

struct PostDag {
  std::vector<PNode> nodes;
  std::map<std::array<int, 6>, int> memo;
  int leaf(int acc_slot) {
    std::array<int, 6> k{-1, acc_slot, 0, 0, 0, 0};
    auto it = memo.find(k);
    if (it != memo.end()) return it->second;
    PNode p;
    p.leaf_slot = acc_slot;
    nodes.push_back(p);
    memo.emplace(k, (int)nodes.size() - 1);
    return (int)nodes.size() - 1;
  }
  int op(int kind, int dir, int n, int s1, int s2, int s3,
         const std::array<int, 6>* key) {
    if (key) {
      auto it = memo.find(*key);
      if (it != memo.end()) return it->second;
    }
    PNode p;
    p.kind = kind;
    p.dir = dir;
    p.n = n;
    p.src[0] = s1;
    p.src[1] = s2;
    p.src[2] = s3;
    nodes.push_back(p);
    const int id = (int)nodes.size() - 1;
    if (key) memo.emplace(*key, id);
    return id;
  }
};

uint32_t slot32(int v) {
  if (v < 0 || v >= (1 << 30)) throw std::runtime_error("lgx: slot index overflow");
  return uint32_t(v);
}

// ASAP levels of the op nodes of a post DAG restricted to `ids`.
template <class N>
int asap_levels(std::vector<N>& nodes) {
  bool changed = true;
  while (changed) {
    changed = false;
    for (auto& n : nodes) {
      if (n.kind < 0) continue;
      int lv = 0;
      for (int s : n.src)
        if (s >= 0 && nodes[s].kind >= 0) lv = std::max(lv, nodes[s].level + 1);
      if (lv != n.level) {
        n.level = lv;
        changed = true;
      }
    }
  }
  int nl = 0;
  for (auto& n : nodes)
    if (n.kind >= 0) nl = std::max(nl, n.level + 1);
  return nl;
}

}  // namespace

int num_classes() {
  int n = 0;
  for (int la = 0; la <= kMaxLInternal; ++la)
    for (int lb = 0; lb <= la; ++lb)
      for (int lc = 0; lc <= kMaxLInternal; ++lc)
        for (int ld = 0; ld <= lc; ++ld)
          if (la + lb <= lc + ld) ++n;
  return n;
}

int class_index(int la, int lb, int lc, int ld) {
  int n = 0;
  for (int a = 0; a <= kMaxLInternal; ++a)
    for (int b = 0; b <= a; ++b)
      for (int c = 0; c <= kMaxLInternal; ++c)
        for (int d = 0; d <= c; ++d)
          if (a + b <= c + d) {
            if (a == la && b == lb && c == lc && d == ld) return n;
            ++n;
          }
  return -1;
}

ClassProgramHost build_class_program(int la, int lb, int lc, int ld, int deriv) {
  if (la < lb || lc < ld || la + lb > lc + ld || la > kMaxLInternal || lc > kMaxLInternal ||
      deriv < 0 || deriv > kMaxDeriv)
    throw std::runtime_error("lgx: non-canonical class");
  ClassProgramHost P;
  P.la = la; P.lb = lb; P.lc = lc; P.ld = ld; P.deriv = deriv;
  const int L = la + lb + lc + ld;
  P.mmax = L + deriv;
  P.nweights = deriv ? 4 : 1;

  // ---- contracted sets: (weight, e-range, f-range)
  struct AccSet { int w, e0, e1, f0, f1; };
  std::vector<AccSet> sets;
  if (!deriv) {
    sets.push_back({0, la, la + lb, lc, lc + ld});
  } else {
    // weight 1: feeds (a-1_i b|, (a b-1_i| and (ab|c d-1_i)
    if (la > 0 || lb > 0 || ld > 0)
      sets.push_back({0, std::max(la - 1, 0), la + lb, lc, lc + ld});
    sets.push_back({1, la + 1, la + lb + 1, lc, lc + ld});  // 2 alpha_A
    sets.push_back({2, la, la + lb + 1, lc, lc + ld});      // 2 alpha_B
    sets.push_back({3, la, la + lb, lc, lc + ld + 1});      // 2 alpha_D
  }
  std::map<std::array<int, 3>, int> acc_slot;  // (w, e, f) -> slot
  int nacc = 0;
  for (const auto& s : sets)
    for (int le = s.e0; le <= s.e1; ++le)
      for (int lf = s.f0; lf <= s.f1; ++lf) {
        if (le + lf > P.mmax) continue;
        for (const C3& e : comps(le))
          for (const C3& f : comps(lf)) acc_slot[{s.w, cidx(e), cidx(f)}] = nacc++;
      }
  P.nacc = nacc;
  auto decode = [](int ci) {
    int l = 0;
    while (cum(l + 1) <= ci) ++l;
    return comps(l)[ci - cum(l)];
  };

  // ---- VRR DAG, levels, slots
  VrrDag dag;
  std::vector<std::pair<int, uint32_t>> accs;  // (node, acc slot | w<<30)
  for (const auto& kv : acc_slot) {
    const int node = dag.get(decode(kv.first[1]), decode(kv.first[2]), 0);
    accs.push_back({node, uint32_t(kv.second) | (uint32_t(kv.first[0]) << 30)});
  }
  auto& nodes = dag.nodes;
  bool changed = true;
  while (changed) {
    changed = false;
    for (auto& n : nodes) {
      if (n.kind < 0) continue;
      int lv = 0;
      for (int s : n.src)
        if (s >= 0) lv = std::max(lv, nodes[s].level + 1);
      if (lv != n.level) {
        n.level = lv;
        changed = true;
      }
    }
  }
  int nlev = 0;
  for (auto& n : nodes) nlev = std::max(nlev, n.level + 1);
  for (auto& n : nodes)
    for (int s : n.src)
      if (s >= 0) nodes[s].last_use = std::max(nodes[s].last_use, n.level);
  for (auto& a : accs)
    nodes[a.first].last_use = std::max(nodes[a.first].last_use, nodes[a.first].level);
  std::vector<std::vector<int>> bylev(nlev);
  for (int i = 0; i < (int)nodes.size(); ++i) bylev[nodes[i].level].push_back(i);
  for (auto& v : bylev)
    std::stable_sort(v.begin(), v.end(), [&](int a, int b) {
      auto shape = [&](const VNode& n) {
        return n.kind * 4 + (n.n1 ? 2 : 0) + (n.ne ? 1 : 0);
      };
      return shape(nodes[a]) < shape(nodes[b]);
    });
  SlotPool pool(nacc);
  P.leaf_slot0 = nacc;
  for (int m = 0; m <= P.mmax; ++m) pool.take();
  std::vector<std::vector<int>> free_after(nlev);
  for (int i = 0; i < (int)nodes.size(); ++i)
    if (nodes[i].last_use >= 0) free_after[nodes[i].last_use].push_back(i);
  P.vrr_lev.push_back(0);
  P.acc_lev.push_back(0);
  for (int k = 0; k < nlev; ++k) {
    for (int id : bylev[k]) {
      VNode& n = nodes[id];
      if (n.kind < 0) {
        if (n.e.l() != 0 || n.f.l() != 0) throw std::runtime_error("lgx: bad leaf");
        n.slot = P.leaf_slot0 + n.m;
      } else {
        n.slot = pool.take();
      }
    }
    if (k > 0)
      for (int id : bylev[k]) {
        const VNode& n = nodes[id];
        auto sl = [&](int s) { return s >= 0 ? slot32(nodes[s].slot) : 0u; };
        // the kernel's factor table holds k/(2 zeta) etc. for k = 0..7
        if (n.n1 > 7 || n.ne > 7) throw std::runtime_error("lgx: recurrence factor out of range");
        P.vrr_ops.push_back(slot32(n.slot));
        for (int t = 0; t < 5; ++t) P.vrr_ops.push_back(sl(n.src[t]));
        P.vrr_ops.push_back(uint32_t(n.kind) | (uint32_t(n.dir) << 1) |
                            (uint32_t(n.n1) << 3) | (uint32_t(n.ne) << 8));
        P.vrr_ops.push_back(0);
        P.vrr_flops += 3 + (n.n1 ? 3 : 0) + (n.ne ? 2 : 0);
      }
    for (auto& a : accs)
      if (nodes[a.first].level == k) {
        P.acc_ops.push_back(a.second & 0x3FFFFFFFu);
        P.acc_ops.push_back(slot32(nodes[a.first].slot) | (a.second & 0xC0000000u));
        P.vrr_flops += 2;
      }
    P.vrr_lev.push_back((int)P.vrr_ops.size() / 8);
    P.acc_lev.push_back((int)P.acc_ops.size() / 2);
    for (int id : free_after[k])
      if (nodes[id].kind >= 0) pool.give(nodes[id].slot);
  }
  const int vrr_work = pool.high;

  // ---- post-contraction program, one phase per output group
  const auto ca = comps(la), cb = comps(lb), cc = comps(lc), cd = comps(ld);
  P.ncart4 = int(ca.size() * cb.size() * cc.size() * cd.size());
  P.nphases = deriv ? 3 : 1;
  P.sets_per_phase = deriv ? 3 : 1;
  const int nout = P.sets_per_phase * P.ncart4;
  P.cart_out = nacc;
  P.cbuf = nacc + nout;
  const int temps0 = P.cbuf + (deriv ? 3 * P.ncart4 : 0);
  P.sph_tmp = temps0;
  int post_high = 0;
  P.post_lev.push_back(0);
  P.phase_lev.push_back(0);
  auto acc_of = [&](int w, const C3& e, const C3& f) {
    auto it = acc_slot.find({w, cidx(e), cidx(f)});
    if (it == acc_slot.end()) throw std::runtime_error("lgx: missing contracted integral");
    return it->second;
  };
  for (int ph = 0; ph < P.nphases; ++ph) {
    PostDag pd;
    std::function<int(int, C3, C3, C3)> bra = [&](int w, C3 a, C3 b, C3 f) -> int {
      if (b.l() == 0) return pd.leaf(acc_of(w, a, f));
      std::array<int, 6> key{0, w, cidx(a), cidx(b), cidx(f), 0};
      auto it = pd.memo.find(key);
      if (it != pd.memo.end()) return it->second;
      const int i = first_dir(b);
      const int s1 = bra(w, shift(a, i, +1), shift(b, i, -1), f);
      const int s2 = bra(w, a, shift(b, i, -1), f);
      return pd.op(kHrrBra, i, 0, s1, s2, -1, &key);
    };
    std::function<int(int, C3, C3, C3, C3)> ket = [&](int w, C3 a, C3 b, C3 c, C3 d) -> int {
      if (d.l() == 0) return bra(w, a, b, c);
      std::array<int, 6> key{1, w, cidx(a), cidx(b), cidx(c), cidx(d)};
      auto it = pd.memo.find(key);
      if (it != pd.memo.end()) return it->second;
      const int j = first_dir(d);
      const int s1 = ket(w, a, b, shift(c, j, +1), shift(d, j, -1));
      const int s2 = ket(w, a, b, c, shift(d, j, -1));
      return pd.op(kHrrKet, j, 0, s1, s2, -1, &key);
    };
    std::vector<int> outputs(nout, -1);
    if (!deriv) {
      int o = 0;
      for (auto& a : ca) for (auto& b : cb) for (auto& c : cc) for (auto& d : cd)
        outputs[o++] = ket(0, a, b, c, d);
    } else {
      // phase 0: centre A (weight 2 alpha_A), 1: B (2 alpha_B), 2: D (2 alpha_D)
      const int ctr = ph == 0 ? 0 : (ph == 1 ? 1 : 3);
      const int wup = ph + 1;
      for (int xyz = 0; xyz < 3; ++xyz) {
        int o = 0;
        for (auto& a : ca) for (auto& b : cb) for (auto& c : cc) for (auto& d : cd) {
          C3 q[4] = {a, b, c, d};
          C3 up[4] = {a, b, c, d};
          up[ctr] = shift(up[ctr], xyz, +1);
          const int su = ket(wup, up[0], up[1], up[2], up[3]);
          const int nn = q[ctr][xyz];
          int sd = -1;
          if (nn > 0) {
            C3 dn[4] = {a, b, c, d};
            dn[ctr] = shift(dn[ctr], xyz, -1);
            sd = ket(0, dn[0], dn[1], dn[2], dn[3]);
          }
          outputs[size_t(xyz) * P.ncart4 + o++] = pd.op(kDeriv, 0, nn, su, sd, -1, nullptr);
        }
      }
    }
    for (int o = 0; o < nout; ++o) {
      int id = outputs[o];
      if (pd.nodes[id].kind < 0 || pd.nodes[id].pinned_slot >= 0) {
        id = pd.op(kCopy, 0, 0, id, -1, -1, nullptr);
        outputs[o] = id;
      }
      pd.nodes[id].pinned_slot = P.cart_out + o;
    }
    auto& pn = pd.nodes;
    const int npl = asap_levels(pn);
    for (auto& n : pn)
      if (n.kind >= 0)
        for (int s : n.src)
          if (s >= 0) pn[s].last_use = std::max(pn[s].last_use, n.level);
    std::vector<std::vector<int>> plev(npl);
    for (int i = 0; i < (int)pn.size(); ++i)
      if (pn[i].kind >= 0) plev[pn[i].level].push_back(i);
    SlotPool ppool(temps0);
    std::vector<std::vector<int>> pfree(npl);
    for (int i = 0; i < (int)pn.size(); ++i)
      if (pn[i].kind >= 0 && pn[i].pinned_slot < 0 && pn[i].last_use >= 0)
        pfree[pn[i].last_use].push_back(i);
    for (int k = 0; k < npl; ++k) {
      for (int id : plev[k]) {
        PNode& n = pn[id];
        n.slot = n.pinned_slot >= 0 ? n.pinned_slot : ppool.take();
      }
      for (int id : plev[k]) {
        const PNode& n = pn[id];
        auto sl = [&](int s) -> uint32_t {
          if (s < 0) return 0u;
          return slot32(pn[s].kind < 0 ? pn[s].leaf_slot : pn[s].slot);
        };
        P.post_ops.push_back(slot32(n.slot));
        P.post_ops.push_back(sl(n.src[0]));
        P.post_ops.push_back(sl(n.src[1]));
        P.post_ops.push_back(uint32_t(n.kind) | (uint32_t(n.dir) << 4) |
                             (uint32_t(n.n) << 8));
        P.post_flops += (n.kind == kCopy) ? 0 : 2;
      }
      P.post_lev.push_back((int)P.post_ops.size() / 4);
      for (int id : pfree[k]) ppool.give(pn[id].slot);
    }
    post_high = std::max(post_high, ppool.high);
    P.phase_lev.push_back((int)P.post_lev.size() - 1);
  }
  const int post_work = (temps0 - nacc) + std::max(post_high, P.ncart4);
  P.nwork = std::max(vrr_work, post_work);
  P.vrr_work = vrr_work;
  slot32(P.nacc + P.nwork);
  return P;
}

}  // namespace lgx
