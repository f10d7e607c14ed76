// sg_host_mesh.cu -- host-side model construction: deck reader, hex2spec,
// face constraints, dof numbering, gather groups and the sparse element-matrix
// layout tables.  Setup-time code; the solve itself runs on the device.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <numeric>
#include <sstream>
#include <thread>

#include "sg_internal.h"

namespace sg {

namespace {

// Local node n = i + 3j + 9k (i along xi fastest) -- the GLL point order of
// gll_quadrature (src/gll_library.f90:46-60) and hex2spec (src/mesh_spec.f90:88-107).
// Exodus faces (src/element.f90:48-141): 1 y-min, 2 x-max, 3 y-max, 4 x-min, 5 z-min, 6 z-max.
bool on_face(int n, int face) {
  int i = n % 3, j = (n / 3) % 3, k = n / 9;
  switch (face) {
    case 1: return j == 0;
    case 2: return i == 2;
    case 3: return j == 2;
    case 4: return i == 0;
    case 5: return k == 0;
    case 6: return k == 2;
  }
  return false;
}

}  // namespace

namespace {
// Host threads for the mesh build (capped: the server may build several meshes at once).
int host_threads() {
  unsigned h = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(h, 16u));
}

template <typename F>
void parallel_ranges(size_t n, int nt, F f) {
  if (nt <= 1 || n < 65536) { f(size_t(0), n); return; }
  std::vector<std::thread> th;
  const size_t step = (n + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    const size_t a = t * step, b = std::min(n, a + step);
    if (a >= b) break;
    th.emplace_back(f, a, b);
  }
  for (auto& x : th) x.join();
}

struct KeyIdx {
  double k;
  int i;
};

// get_global's ordering (src/mesh_spec.f90:146-262): three passes, x then y
// then z.  Each pass stable-sorts every current segment by that coordinate
// and then starts a new segment wherever the coordinate jumps by more than tol
// from its predecessor.  The first pass is one segment, sorted as stable-sorted
// chunks joined by stable merges; the later passes sort their segments
// independently.  Stability at every step keeps the order exactly that of one
// sequential stable sort per segment.
void merge_order(const std::vector<double>* keys[3], size_t np, double tol, std::vector<int>& order,
                 std::vector<char>& seg) {
  const int nt = host_threads();
  order.resize(np);
  std::iota(order.begin(), order.end(), 0);
  seg.assign(np, 0);
  if (np == 0) return;
  seg[0] = 1;
  auto less = [](const KeyIdx& p, const KeyIdx& q) { return p.k < q.k; };
  std::vector<KeyIdx> buf(np), tmp;
  for (int d = 0; d < 3; ++d) {
    const std::vector<double>& key = *keys[d];
    parallel_ranges(np, nt, [&](size_t a, size_t b) {
      for (size_t i = a; i < b; ++i) buf[i] = {key[order[i]], order[i]};
    });
    if (d == 0) {
      const int nc = (int)std::max<size_t>(1, std::min<size_t>((size_t)nt, np / 65536));
      std::vector<size_t> cut(nc + 1);
      for (int c = 0; c <= nc; ++c) cut[c] = np * c / nc;
      {
        std::vector<std::thread> th;
        for (int c = 0; c < nc; ++c)
          th.emplace_back([&, c] { std::stable_sort(buf.begin() + cut[c], buf.begin() + cut[c + 1], less); });
        for (auto& x : th) x.join();
      }
      tmp.resize(np);
      while (cut.size() > 2) {
        std::vector<size_t> nx;
        std::vector<std::thread> th;
        size_t c = 0;
        for (; c + 2 < cut.size(); c += 2) {
          const size_t a = cut[c], m = cut[c + 1], b = cut[c + 2];
          th.emplace_back([&, a, m, b] {
            std::merge(buf.begin() + a, buf.begin() + m, buf.begin() + m, buf.begin() + b, tmp.begin() + a, less);
          });
          nx.push_back(a);
        }
        if (c + 1 < cut.size()) {  // an unpaired last chunk is carried over
          std::copy(buf.begin() + cut[c], buf.begin() + cut[c + 1], tmp.begin() + cut[c]);
          nx.push_back(cut[c]);
        }
        nx.push_back(np);
        for (auto& x : th) x.join();
        std::swap(buf, tmp);
        cut.swap(nx);
      }
    } else {
      std::vector<size_t> starts;
      for (size_t i = 0; i < np; ++i)
        if (seg[i]) starts.push_back(i);
      starts.push_back(np);
      const size_t ns = starts.size() - 1;
      parallel_ranges(ns, nt, [&](size_t a, size_t b) {
        for (size_t u = a; u < b; ++u)
          if (starts[u + 1] - starts[u] > 1) std::stable_sort(buf.begin() + starts[u], buf.begin() + starts[u + 1], less);
      });
    }
    parallel_ranges(np, nt, [&](size_t a, size_t b) {
      for (size_t i = a; i < b; ++i) order[i] = buf[i].i;
      for (size_t i = std::max<size_t>(a, 1); i < b; ++i)
        if (std::fabs(buf[i].k - buf[i - 1].k) > tol) seg[i] = 1;
    });
  }
}
}  // namespace

// hex2spec (src/mesh_spec.f90:17-143): GLL point coordinates from the
// trilinear hex8 map, duplicate points merged with the reference's
// lexicographic tolerance test (get_global, src/mesh_spec.f90:146-262), nodes
// renumbered in first-touch order over (element, k, j, i)
// (get_global_indirect_addressing, src/mesh_spec.f90:357-386).  A point's
// coordinates are those of the last element that touches it, as in the
// reference's overwrite loop.
bool hex2spec(HostMesh& M, int nnode8, const double* x8, const double* y8, const double* z8,
              const int* conn8, std::string& err) {
  const int nelmt = M.nelmt;
  const double xi[3] = {-1.0, 0.0, 1.0};
  double shape[8][NGLL];
  const double e8 = 0.125;
  int n = 0;
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i, ++n) {
        double xp = 1 + xi[i], xm = 1 - xi[i], ep = 1 + xi[j], em = 1 - xi[j], zp = 1 + xi[k], zm = 1 - xi[k];
        shape[0][n] = e8 * xm * em * zm; shape[1][n] = e8 * xp * em * zm;
        shape[2][n] = e8 * xp * ep * zm; shape[3][n] = e8 * xm * ep * zm;
        shape[4][n] = e8 * xm * em * zp; shape[5][n] = e8 * xp * em * zp;
        shape[6][n] = e8 * xp * ep * zp; shape[7][n] = e8 * xm * ep * zp;
      }
  double xmin = x8[0], xmax = x8[0];
  for (int i = 0; i < nnode8; ++i) { xmin = std::min(xmin, x8[i]); xmax = std::max(xmax, x8[i]); }
  const size_t np = (size_t)nelmt * NGLL;
  for (size_t t = 0; t < (size_t)nelmt * 8; ++t)
    if (conn8[t] < 1 || conn8[t] > nnode8) { err = "ERROR: connectivity references a node out of range!"; return false; }
  std::vector<double> xs(np), ys(np), zs(np);
  parallel_ranges((size_t)nelmt, host_threads(), [&](size_t e0, size_t e1) {
    for (size_t e = e0; e < e1; ++e) {
      int c[8];
      for (int g = 0; g < 8; ++g) c[g] = conn8[e * 8 + g] - 1;
      for (int p = 0; p < NGLL; ++p) {
        double xg = 0, yg = 0, zg = 0;
        for (int g = 0; g < 8; ++g) {
          xg = xg + shape[g][p] * x8[c[g]];
          yg = yg + shape[g][p] * y8[c[g]];
          zg = zg + shape[g][p] * z8[c[g]];
        }
        const size_t q = e * NGLL + p;
        xs[q] = xg; ys[q] = yg; zs[q] = zg;
      }
    }
  });
  // Merge: order points by (x, y, z) with the reference's segment-by-segment
  // tolerance scheme; a new point starts where any coordinate jumps by more
  // than tol relative to the previous point in the final order.
  const double tol = 1.e-10 * std::fabs(xmax - xmin);
  std::vector<int> order;
  std::vector<char> seg;
  const std::vector<double>* keys[3] = {&xs, &ys, &zs};
  merge_order(keys, np, tol, order, seg);
  std::vector<int> iglob(np);
  int ig = 0;
  for (size_t i = 0; i < np; ++i) {
    if (seg[i]) ++ig;
    iglob[order[i]] = ig - 1;
  }
  std::vector<int> mask(ig, -1);
  int num = 0;
  M.g_num.assign(np, 0);
  for (size_t i = 0; i < np; ++i) {
    int o = iglob[i];
    if (mask[o] < 0) mask[o] = num++;
    M.g_num[i] = mask[o];
  }
  M.nnode = num;
  M.g_coord.assign((size_t)3 * num, 0.0);
  for (size_t i = 0; i < np; ++i) {
    int nd = M.g_num[i];
    M.g_coord[(size_t)3 * nd + 0] = xs[i];
    M.g_coord[(size_t)3 * nd + 1] = ys[i];
    M.g_coord[(size_t)3 * nd + 2] = zs[i];
  }
  return true;
}

// apply_bc (src/apply_bc.f90:7-143): every listed (element, face) fixes its
// face nodes in that direction; free dofs are numbered node-major.
bool apply_bc(HostMesh& M, const int* bc_counts, const int* bc_pairs, std::string& err) {
  M.gdof.assign((size_t)3 * M.nnode, 1);
  size_t off = 0;
  for (int d = 0; d < 3; ++d)
    for (int i = 0; i < bc_counts[d]; ++i, ++off) {
      int e = bc_pairs[2 * off] - 1, f = bc_pairs[2 * off + 1];
      if (e < 0 || e >= M.nelmt || f < 1 || f > 6) { err = "ERROR: bad element/face in a BC list!"; return false; }
      for (int a = 0; a < NGLL; ++a)
        if (on_face(a, f)) M.gdof[(size_t)3 * M.g_num[(size_t)e * NGLL + a] + d] = 0;
    }
  int neq = 0;
  for (int j = 0; j < M.nnode; ++j)
    for (int i = 0; i < 3; ++i)
      if (M.gdof[(size_t)3 * j + i] != 0) M.gdof[(size_t)3 * j + i] = ++neq;
  M.neq = neq;
  return true;
}

// gdof_elmt(:,e) = reshape(gdof(:,g_num(:,e)),(/nedof/)) (src/slope.F90:140-144)
void build_gdof_elmt(HostMesh& M) {
  M.gdof_elmt.assign((size_t)NEDOF * M.nelmt, 0);
  for (int e = 0; e < M.nelmt; ++e)
    for (int a = 0; a < NGLL; ++a)
      for (int d = 0; d < 3; ++d)
        M.gdof_elmt[(size_t)e * NEDOF + 3 * a + d] = M.gdof[(size_t)3 * M.g_num[(size_t)e * NGLL + a] + d];
}

// Gather groups from the element dof map.  A node is identified by its
// smallest non-zero dof number (the same in every element that holds it);
// nodes whose three dofs are fixed receive nothing and are skipped.
// Counting sort by that key keeps slots in increasing element order.
void build_groups_from_gdof(const int* ge, int nelmt, int neq, GatherTopo& T) {
  std::vector<int> key((size_t)nelmt * NGLL);
  std::vector<int> cnt(neq + 2, 0);
  for (size_t s = 0; s < (size_t)nelmt * NGLL; ++s) {
    const int* g = ge + 3 * s;
    int k = 0;
    for (int d = 0; d < 3; ++d)
      if (g[d] > 0 && (k == 0 || g[d] < k)) k = g[d];
    key[s] = k;
    if (k) cnt[k]++;
  }
  // groups are the keys that occur, in increasing key order
  std::vector<int> gid(neq + 2, -1);
  int ng = 0;
  for (int k = 1; k <= neq; ++k)
    if (cnt[k]) gid[k] = ng++;
  T.ngroups = ng;
  T.ptr.assign(ng + 1, 0);
  for (int k = 1; k <= neq; ++k)
    if (cnt[k]) T.ptr[gid[k] + 1] = cnt[k];
  for (int g = 0; g < ng; ++g) T.ptr[g + 1] += T.ptr[g];
  T.ent.assign(T.ptr[ng], 0);
  T.dof.assign((size_t)3 * ng, 0);
  T.pos.assign((size_t)nelmt * NGLL, -1);
  std::vector<int> fill(T.ptr.begin(), T.ptr.end() - 1);
  for (size_t s = 0; s < (size_t)nelmt * NGLL; ++s) {
    int k = key[s];
    if (!k) continue;
    int g = gid[k];
    T.pos[s] = fill[g];
    T.ent[fill[g]++] = (int)s;
    for (int d = 0; d < 3; ++d) T.dof[(size_t)3 * g + d] = ge[3 * s + d];
  }
}

// Sparse symmetric element-matrix layout (see KS_NNZ in sg_internal.h).
const KsTables& ks_tables() {
  static KsTables T;
  static bool init = false;
  if (init) return T;
  auto coupled = [](int n, int m) {
    int dn = (n % 3 != m % 3) + ((n / 3) % 3 != (m / 3) % 3) + (n / 9 != m / 9);
    return dn <= 2;
  };
  int off[NGLL][NGLL];
  int o = 0, ne = 0;
  for (int m = 0; m < NGLL; ++m)
    for (int n = 0; n <= m; ++n) {
      off[n][m] = -1;
      if (!coupled(n, m)) continue;
      off[n][m] = o;
      for (int c = 0; c < 3; ++c)
        for (int d = 0; d < 3; ++d) T.entry[ne++] = (3 * n + c) | ((3 * m + d) << 8);
      o += 9;
    }
  for (int n = 0; n < NGLL; ++n) {
    int s = 0;
    for (int m = 0; m < NGLL; ++m) {
      if (!coupled(n, m)) continue;
      int kind = (n == m) ? 0 : (n < m ? 1 : 2);
      int of = (n <= m) ? off[n][m] : off[m][n];
      T.nbr[n][s++] = m | (kind << 5) | (of << 8);
    }
  }
  init = true;
  return T;
}

// ---------------------------------------------------------------------------
// .sem deck reader: the subset of src/read_input.f90:13-619 the solve path
// uses (preinfo, mesh, bc, material, control, stress0, eqload, water; save and
// traction lines are accepted and ignored).  File names resolve relative to the
// deck's directory.  Defaults: cg_tol = nl_tol = 1e-12, cg_maxiter =
// nl_maxiter = 100 (src/read_input.f90:109-110).
// ---------------------------------------------------------------------------
namespace {
std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? "" : s.substr(a, b - a + 1);
}
std::string unquote(std::string v) {
  v = trim(v);
  if (v.size() >= 2 && (v[0] == '\'' || v[0] == '"')) v = v.substr(1, v.size() - 2);
  return v;
}
}  // namespace

bool read_deck(const char* path, HostMesh& M, std::vector<double>& x8, std::vector<double>& y8,
               std::vector<double>& z8, std::vector<int>& conn, std::vector<int>& mid,
               std::vector<double>& props, std::vector<int>& bc_counts, std::vector<int>& bc_pairs,
               std::string& err) {
  std::ifstream in(path);
  if (!in) { err = std::string("ERROR: input file \"") + path + "\" cannot be opened!"; return false; }
  std::string sp(path);
  size_t sl = sp.find_last_of('/');
  std::string base = (sl == std::string::npos) ? "./" : sp.substr(0, sl + 1);
  std::map<std::string, std::map<std::string, std::string>> L;
  std::string line;
  while (std::getline(in, line)) {
    std::string t = trim(line);
    if (t.empty() || t[0] == '#') continue;
    while (!t.empty() && t.back() == '&') {
      t.pop_back();
      std::string nx;
      if (!std::getline(in, nx)) { err = "ERROR: line continuation incomplete!"; return false; }
      t += trim(nx);
    }
    size_t s = t.find(' ');
    std::string token = t.substr(0, s), rest = s == std::string::npos ? "" : t.substr(s + 1);
    static const char* known[] = {"preinfo:", "mesh:", "bc:", "stress0:", "traction:", "material:",
                                  "eqload:", "water:", "control:", "save:"};
    bool ok = false;
    for (const char* k : known) ok = ok || token == k;
    if (!ok) { err = "ERROR: invalid line type: \"" + token + "\"!"; return false; }
    if (L.count(token)) { err = "ERROR: copy of line type " + token + " not permitted!"; return false; }
    auto& kv = L[token];
    std::stringstream ss(rest);
    std::string arg;
    while (std::getline(ss, arg, ',')) {
      size_t eq = arg.find('=');
      if (eq != std::string::npos) kv[trim(arg.substr(0, eq))] = unquote(arg.substr(eq + 1));
    }
  }
  // required lines, with the reference's messages (src/read_input.f90:409-442)
  static const char* need[][2] = {{"preinfo:", "pre"}, {"mesh:", "mesh"}, {"bc:", "BC"},
                                  {"material:", "material"}, {"control:", "control"}};
  for (auto& nd : need)
    if (!L.count(nd[0])) {
      err = std::string("ERROR: cannot read ") + nd[1] + " information! make sure the line with \"" + nd[0] +
            "\" token is correct.";
      return false;
    }
  auto& pre = L["preinfo:"];
  {  // method defaults to sem and a blank value keeps it (src/read_input.f90:87,161-162,173-180)
    const std::string method = (pre.count("method") && !trim(pre["method"]).empty()) ? trim(pre["method"]) : "sem";
    // the reference accepts fem; this solve path is spectral only (a
    // limitation of this library, not a reference message)
    if (method == "fem") { err = "ERROR: method='fem' is not supported by this solver (method='sem' only)!"; return false; }
    if (method != "sem") { err = "ERROR: wrong value for method!"; return false; }
  }
  if (pre["ngllx"] != "3" || pre["nglly"] != "3" || pre["ngllz"] != "3") {
    err = "ERROR: only ngllx=nglly=ngllz=3 is supported!"; return false;
  }
  auto& mesh = L["mesh:"];
  std::vector<double>* xyz[3] = {&x8, &y8, &z8};
  const char* cf[3] = {"xfile", "yfile", "zfile"};
  int nnode8 = -1;
  for (int d = 0; d < 3; ++d) {
    std::ifstream f(base + mesh[cf[d]]);
    int n;
    if (!f || !(f >> n)) { err = "ERROR: file \"" + mesh[cf[d]] + "\" cannot be opened!"; return false; }
    if (nnode8 >= 0 && n != nnode8) { err = "ERROR: total number of nodes mismatch!"; return false; }
    nnode8 = n;
    xyz[d]->resize(n);
    for (int i = 0; i < n; ++i) f >> (*xyz[d])[i];
  }
  {
    std::ifstream f(base + mesh["confile"]);
    if (!f || !(f >> M.nelmt)) { err = "ERROR: connectivity file cannot be opened!"; return false; }
    conn.resize((size_t)8 * M.nelmt);
    for (auto& c : conn) f >> c;
  }
  {
    std::ifstream f(base + mesh["idfile"]);
    int n;
    if (!f || !(f >> n)) { err = "ERROR: material id file cannot be opened!"; return false; }
    if (n != M.nelmt) { err = "ERROR: total number of elements mismatch!"; return false; }
    mid.resize(n);
    for (auto& m : mid) f >> m;
  }
  {
    auto& mat = L["material:"];
    std::ifstream f(base + mat["matfile"]);
    if (!f) { err = "ERROR: material list cannot be opened!"; return false; }
    std::string l;
    std::getline(f, l);
    std::getline(f, l);
    M.nmatblk = std::atoi(trim(l).c_str());
    props.assign((size_t)6 * M.nmatblk, 0.0);
    for (int i = 0; i < M.nmatblk; ++i) {
      std::getline(f, l);
      for (char& ch : l) if (ch == ',') ch = ' ';
      std::stringstream ss(l);
      int id, dom, typ;
      ss >> id >> dom >> typ;
      if (typ != 0) { err = "ERROR: only type_blk 0 material blocks are supported!"; return false; }
      for (int k = 0; k < 6; ++k) ss >> props[(size_t)6 * i + k];
    }
    M.allelastic = mat.count("allelastic") && std::atoi(mat["allelastic"].c_str()) == 1;
    for (int m : mid)
      if (m < 1 || m > M.nmatblk) { err = "ERROR: material IDs must be consistent with the defined material regions!"; return false; }
    if (L.count("water:")) {  // src/read_input.f90:307-317 and 602-611
      M.iswater = 1;
      M.wsfile = base + L["water:"]["wsfile"];
      int nwmat;
      if (!(f >> nwmat)) { err = "ERROR: water IDs cannot be read from material list!"; return false; }
      M.water_ids.resize(nwmat > 0 ? nwmat : 0);
      for (auto& id : M.water_ids)
        if (!(f >> id) || id < 1 || id > M.nmatblk) { err = "ERROR: water IDs cannot be read from material list!"; return false; }
    }
  }
  bc_counts.assign(3, 0);
  bc_pairs.clear();
  {
    auto& bc = L["bc:"];
    const char* bf[3] = {"uxfile", "uyfile", "uzfile"};
    for (int d = 0; d < 3; ++d) {
      std::ifstream f(base + bc[bf[d]]);
      if (!f) { err = "ERROR: file \"" + bc[bf[d]] + "\" cannot be opened!"; return false; }
      int bctype;
      double val;
      while (f >> bctype >> val) {
        // the reference's checks and messages (src/apply_bc.f90:36-60)
        if (val != 0.0) { err = "ERROR: nonzero displacement BC not implemented!"; return false; }
        if (bctype == 0) { err = "ERROR: nodal displacement BC not implemented!"; return false; }
        if (bctype == 1) { err = "ERROR: edge displacement BC not implemented!"; return false; }
        if (bctype != 2) { err = "ERROR: undefined displacement BC type ux! " + std::to_string(bctype); return false; }
        int nel;
        f >> nel;
        for (int i = 0; i < nel; ++i) {
          int e, fc;
          f >> e >> fc;
          bc_pairs.push_back(e);
          bc_pairs.push_back(fc);
          bc_counts[d]++;
        }
      }
    }
  }
  // bc lists are read per direction; regroup as ux list, uy list, uz list (already in that order)
  auto& ctl = L["control:"];
  if (ctl.count("cg_tol")) M.cg_tol = std::atof(ctl["cg_tol"].c_str());
  if (ctl.count("cg_maxiter")) M.cg_maxiter = std::atoi(ctl["cg_maxiter"].c_str());
  if (ctl.count("nl_tol")) M.nl_tol = std::atof(ctl["nl_tol"].c_str());
  if (ctl.count("nl_maxiter")) M.nl_maxiter = std::atoi(ctl["nl_maxiter"].c_str());
  if (ctl.count("phinu")) M.phinu = std::atoi(ctl["phinu"].c_str()) == 1;
  if (ctl.count("ninc")) M.ninc = std::atoi(ctl["ninc"].c_str());
  int nsrf = ctl.count("nsrf") ? std::atoi(ctl["nsrf"].c_str()) : 1;
  M.srf.assign(nsrf, 1.0);
  if (ctl.count("srf")) {
    std::stringstream ss(ctl["srf"]);
    for (int i = 0; i < nsrf; ++i)
      if (!(ss >> M.srf[i])) {
        if (nsrf > 1) { err = "ERROR: argument \"srf\" not found or insufficient list for \"srf\"!"; return false; }
      }
  }
  for (double s : M.srf)
    if (s <= 0) { err = "ERROR: \"srf\" must be positive!"; return false; }
  if (ctl.count("nexcav")) {
    M.nexcav = std::atoi(ctl["nexcav"].c_str());
    M.nexcavid.assign(M.nexcav, 1);
    if (ctl.count("nexcavid")) {
      std::stringstream ss(ctl["nexcavid"]);
      for (auto& v : M.nexcavid) ss >> v;
    }
    int tot = 0;
    for (int v : M.nexcavid) tot += v;
    M.excavid.assign(tot, 0);
    std::stringstream ss(ctl["excavid"]);
    for (auto& v : M.excavid) ss >> v;
  }
  if (nsrf > 1 && M.nexcav > 1) { err = "ERROR: cannot run slope stabiliy and excavation simultaneously!"; return false; }
  if (L.count("stress0:")) {
    auto& s0 = L["stress0:"];
    M.s0_type = s0.count("type") ? std::atoi(s0["type"].c_str()) : 0;
    if (s0.count("z0")) M.z0 = std::atof(s0["z0"].c_str());
    if (s0.count("s0")) M.s0 = std::atof(s0["s0"].c_str());
    if (s0.count("k0")) M.k0 = std::atof(s0["k0"].c_str());
  }
  if (L.count("eqload:")) {  // src/read_input.f90:293-303
    auto& eq = L["eqload:"];
    M.iseqload = 1;
    M.eqkx = eq.count("eqkx") ? std::atof(eq["eqkx"].c_str()) : 0.0;
    M.eqky = eq.count("eqky") ? std::atof(eq["eqky"].c_str()) : 0.0;
    M.eqkz = eq.count("eqkz") ? std::atof(eq["eqkz"].c_str()) : 0.0;
  }
  (void)nnode8;
  return true;
}

// Water-surface file (src/compute_pressure.f90:55-86), list-directed: nwsurf,
// then per surface its kind and, by kind, "rdir rx1 rx2 z1" (0),
// "rdir rx1 rx2 z1 z2" (1) or "nface" followed by nface "ielmt iface" lines (2).
bool read_wsfile(const std::string& path, int nelmt, std::vector<WaterSurface>& surf, std::vector<int>& face,
                 std::string& err) {
  std::ifstream in(path);
  if (!in) { err = "ERROR: input file \"" + path + "\" cannot be opened!"; return false; }
  std::stringstream ss;
  {
    std::string all((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    for (char& ch : all) if (ch == ',') ch = ' ';
    ss.str(all);
  }
  int nw;
  if (!(ss >> nw) || nw < 0) { err = "ERROR: bad water-surface file!"; return false; }
  surf.assign(nw, WaterSurface{0, 1, 0, 0, 0.0, 0.0, 0.0, 0.0});
  face.clear();
  for (auto& w : surf) {
    if (!(ss >> w.stype)) { err = "ERROR: bad water-surface file!"; return false; }
    bool ok = true;
    if (w.stype == 0) ok = bool(ss >> w.rdir >> w.rx1 >> w.rx2 >> w.z1);
    else if (w.stype == 1) ok = bool(ss >> w.rdir >> w.rx1 >> w.rx2 >> w.z1 >> w.z2);
    else if (w.stype == 2) {
      ok = bool(ss >> w.nface) && w.nface >= 0;
      w.face0 = (int)face.size() / 2;
      for (int f = 0; ok && f < w.nface; ++f) {
        int e, fc;
        ok = bool(ss >> e >> fc) && e >= 1 && e <= nelmt && fc >= 1 && fc <= 6;
        face.push_back(e - 1);
        face.push_back(fc);
      }
    } else {
      // the reference reads no parameters for other kinds and never matches them
      w.nface = 0;
      w.stype = 3;
    }
    if (!ok || ((w.stype == 0 || w.stype == 1) && (w.rdir < 1 || w.rdir > 3))) {
      err = "ERROR: bad water-surface file!";
      return false;
    }
  }
  return true;
}

}  // namespace sg

// ---------------------------------------------------------------------------
// Host-only mesh handle: the deck reader and mesh builder of
// sg_model_from_deck without any device work (read_input, hex2spec and
// apply_bc: src/read_input.f90:13-619, src/mesh_spec.f90:17-386,
// src/apply_bc.f90:7-143).
// ---------------------------------------------------------------------------
struct sg_mesh {
  sg::HostMesh H;
  std::vector<double> props;  // nmatblk x [gamma E nu phi c psi]
};

namespace {
void mesh_tag(char* errtag, const std::string& m) {
  if (!errtag) return;
  std::memset(errtag, ' ', SG_ERRTAG_LEN);
  std::memcpy(errtag, m.data(), std::min<size_t>(m.size(), SG_ERRTAG_LEN));
}
}  // namespace

extern "C" {

sg_mesh* sg_mesh_from_deck(const char* path, char* errtag) {
  mesh_tag(errtag, "ERROR: unknown!");
  if (!path) return nullptr;
  sg_mesh* m = new sg_mesh();
  sg::HostMesh& H = m->H;
  std::vector<double> x8, y8, z8;
  std::vector<int> conn, mid, cnt, pairs;
  std::string err;
  if (!sg::read_deck(path, H, x8, y8, z8, conn, mid, m->props, cnt, pairs, err)) {
    mesh_tag(errtag, err);
    delete m;
    return nullptr;
  }
  H.mat_id = mid;
  for (int i = 0; i < H.nmatblk; ++i) {
    const double* p = &m->props[(size_t)6 * i];
    H.gam.push_back(p[0]); H.ym.push_back(p[1]); H.nu.push_back(p[2]);
    H.phi.push_back(p[3]); H.coh.push_back(p[4]); H.psi.push_back(p[5]);
  }
  if (!sg::hex2spec(H, (int)x8.size(), x8.data(), y8.data(), z8.data(), conn.data(), err) ||
      !sg::apply_bc(H, cnt.data(), pairs.data(), err)) {
    mesh_tag(errtag, err);
    delete m;
    return nullptr;
  }
  sg::build_gdof_elmt(H);
  mesh_tag(errtag, "");
  return m;
}

void sg_mesh_free(sg_mesh* m) { delete m; }

int sg_mesh_info(const sg_mesh* m, int* info) {
  if (!m || !info) return SG_ERR_BADARG;
  const sg::HostMesh& h = m->H;
  info[0] = h.nnode; info[1] = h.nelmt; info[2] = h.neq; info[3] = h.nmatblk;
  info[4] = (int)h.srf.size(); info[5] = h.nexcav; info[6] = h.iswater; info[7] = (int)h.water_ids.size();
  return SG_OK;
}

int sg_mesh_arrays(const sg_mesh* m, double* g_coord, int* g_num, int* gdof, int* gdof_elmt, int* mat_id,
                   double* props) {
  if (!m) return SG_ERR_BADARG;
  const sg::HostMesh& h = m->H;
  if (g_coord) std::memcpy(g_coord, h.g_coord.data(), sizeof(double) * h.g_coord.size());
  if (g_num) std::memcpy(g_num, h.g_num.data(), sizeof(int) * h.g_num.size());
  if (gdof) std::memcpy(gdof, h.gdof.data(), sizeof(int) * h.gdof.size());
  if (gdof_elmt) std::memcpy(gdof_elmt, h.gdof_elmt.data(), sizeof(int) * h.gdof_elmt.size());
  if (mat_id) std::memcpy(mat_id, h.mat_id.data(), sizeof(int) * h.mat_id.size());
  if (props) std::memcpy(props, m->props.data(), sizeof(double) * m->props.size());
  return SG_OK;
}

int sg_mesh_control(const sg_mesh* m, double* dctl, int* ictl, double* srf, int* nexcavid, int* excavid,
                    int* water_ids) {
  if (!m) return SG_ERR_BADARG;
  const sg::HostMesh& h = m->H;
  if (dctl) {
    const double v[8] = {h.cg_tol, h.nl_tol, h.z0, h.s0, h.k0, h.eqkx, h.eqky, h.eqkz};
    std::memcpy(dctl, v, sizeof(v));
  }
  if (ictl) {
    const int v[8] = {h.cg_maxiter, h.nl_maxiter, h.phinu, h.allelastic, h.nexcav, h.ninc, h.s0_type, h.iseqload};
    std::memcpy(ictl, v, sizeof(v));
  }
  if (srf) std::memcpy(srf, h.srf.data(), sizeof(double) * h.srf.size());
  if (nexcavid) std::memcpy(nexcavid, h.nexcavid.data(), sizeof(int) * h.nexcavid.size());
  if (excavid) std::memcpy(excavid, h.excavid.data(), sizeof(int) * h.excavid.size());
  if (water_ids) std::memcpy(water_ids, h.water_ids.data(), sizeof(int) * h.water_ids.size());
  return SG_OK;
}

}  // extern "C"
