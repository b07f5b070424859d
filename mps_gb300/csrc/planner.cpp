// Sector planner (see planner.hpp).  Every routine restates the bookkeeping of one reference
// function and says which; the device kernels only ever execute the task lists built here.
#include "planner.hpp"

#include <algorithm>
#include <cstring>
#include <map>
#include <numeric>
#include <sstream>

namespace mpsg {

static void fail(int code, const std::string& m) { throw Error(code, m); }

// ------------------------------------------------------------------------------------------
// Spaces (src/vspace.jl)
// ------------------------------------------------------------------------------------------
int64_t Space::dim(int c) const {
  auto it = std::lower_bound(ch.begin(), ch.end(), c);
  if (it == ch.end() || *it != c) return 0;
  return dm[it - ch.begin()];
}

int64_t Space::total() const { return std::accumulate(dm.begin(), dm.end(), (int64_t)0); }

Space Space::make(std::vector<std::pair<int, int64_t>> pairs, bool dual) {
  std::sort(pairs.begin(), pairs.end());
  Space V;
  V.dual = dual;
  for (size_t i = 0; i < pairs.size(); ++i) {
    if (i && pairs[i].first == pairs[i - 1].first) fail(kErrSpaceMismatch, "duplicate charges!");
    if (pairs[i].second <= 0) fail(kErrSpaceMismatch, "space dimension can only be positive!");
    V.ch.push_back(pairs[i].first);
    V.dm.push_back(pairs[i].second);
  }
  return V;
}

Space dual_space(const Space& V) {
  Space W = V;
  W.dual = !V.dual;
  return W;
}

bool isdual_pair(const Space& a, const Space& b) {
  return a.ch == b.ch && a.dm == b.dm && a.dual != b.dual;
}

Space fuse(bool dual, const std::vector<Space>& Vs) {
  const size_t N = Vs.size();
  if (N == 0) fail(kErrArgument, "fuse of no spaces");
  if (N < 2) {
    if (dual == Vs[0].dual) return Vs[0];
    // dual(mapcharges(inv, V)) (vspace.jl:114-117)
    std::vector<std::pair<int, int64_t>> p;
    for (int i = 0; i < Vs[0].size(); ++i) p.push_back({-Vs[0].ch[i], Vs[0].dm[i]});
    Space W = Space::make(p, Vs[0].dual);
    W.dual = !W.dual;
    return W;
  }
  if (N > 2) {
    std::vector<Space> head(Vs.begin(), Vs.end() - 2);
    head.push_back(fuse(dual, std::vector<Space>(Vs.end() - 2, Vs.end())));
    return fuse(dual, head);
  }
  std::map<int, int64_t> acc;
  for (int j = 0; j < Vs[1].size(); ++j) {
    int e2 = eff(Vs[1].ch[j], Vs[1].dual);
    for (int i = 0; i < Vs[0].size(); ++i) {
      int e1 = eff(Vs[0].ch[i], Vs[0].dual);
      int c = dual ? -(e1 + e2) : e1 + e2;
      acc[c] += Vs[0].dm[i] * Vs[1].dm[j];
    }
  }
  Space W;
  W.dual = dual;
  for (auto& kv : acc) {
    W.ch.push_back(kv.first);
    W.dm.push_back(kv.second);
  }
  return W;
}

// ------------------------------------------------------------------------------------------
// Sectors (src/sector.jl)
// ------------------------------------------------------------------------------------------
bool sector_less(const int* a, const int* b, int N) {
  for (int k = N - 1; k >= 0; --k) {
    if (a[k] < b[k]) return true;
    if (a[k] > b[k]) return false;
  }
  return false;
}

static void allsectors_rec(int charge, const std::vector<Space>& Vs, int N,
                           std::vector<int>& lab, std::vector<int64_t>& sz, int Ntot,
                           int* cur_lab, int64_t* cur_sz) {
  if (N == 1) {
    int c = eff(charge, Vs[0].dual);
    int64_t d = Vs[0].dim(c);
    if (d > 0) {
      cur_lab[0] = c;
      cur_sz[0] = d;
      lab.insert(lab.end(), cur_lab, cur_lab + Ntot);
      sz.insert(sz.end(), cur_sz, cur_sz + Ntot);
    }
    return;
  }
  const Space& V = Vs[N - 1];
  for (int i = 0; i < V.size(); ++i) {
    cur_lab[N - 1] = V.ch[i];
    cur_sz[N - 1] = V.dm[i];
    allsectors_rec(charge - eff(V.ch[i], V.dual), Vs, N - 1, lab, sz, Ntot, cur_lab, cur_sz);
  }
}

SectorList allsectorsandsizes(int charge, const std::vector<Space>& Vs) {
  SectorList out;
  out.N = (int)Vs.size();
  if (out.N == 0) return out;
  if (out.N > kMaxLegs) fail(kErrArgument, "too many legs");
  int cl[kMaxLegs];
  int64_t cs[kMaxLegs];
  allsectors_rec(charge, Vs, out.N, out.lab, out.sz, out.N, cl, cs);
  return out;
}

long TensorMeta::find(const int* labels) const {
  const int n = N();
  long lo = 0, hi = (long)nblocks();
  while (lo < hi) {
    long mid = (lo + hi) / 2;
    if (sector_less(sec.labels(mid), labels, n)) lo = mid + 1;
    else hi = mid;
  }
  if (lo < (long)nblocks() && std::equal(labels, labels + n, sec.labels(lo))) return lo;
  return -1;
}

static void finalize_offsets(TensorMeta& m) {
  m.off.resize(m.nblocks());
  int64_t p = 0;
  for (size_t i = 0; i < m.nblocks(); ++i) {
    m.off[i] = p;
    p += m.sec.numel(i);
  }
  m.total = p;
}

TensorMeta TensorMeta::build(int charge, std::vector<Space> space) {
  TensorMeta m;
  m.charge = charge;
  m.space = std::move(space);
  m.sec = allsectorsandsizes(charge, m.space);
  finalize_offsets(m);
  return m;
}

bool same_meta(const TensorMeta& a, const TensorMeta& b) {
  return a.charge == b.charge && a.space == b.space;
}

std::string meta_key(const TensorMeta& m) {
  std::ostringstream os;
  os << m.charge << '|';
  for (auto& V : m.space) {
    os << (V.dual ? 'd' : 'n');
    for (int i = 0; i < V.size(); ++i) os << V.ch[i] << ':' << V.dm[i] << ',';
    os << ';';
  }
  return os.str();
}

// Stable sort of indices by a sector key (Julia's sortperm is stable).
static std::vector<size_t> stable_sortperm(const std::vector<int>& keys, int N) {
  std::vector<size_t> p(keys.size() / (N ? N : 1));
  std::iota(p.begin(), p.end(), 0);
  std::stable_sort(p.begin(), p.end(), [&](size_t a, size_t b) {
    return sector_less(keys.data() + a * N, keys.data() + b * N, N);
  });
  return p;
}

static void colmajor_strides(const int64_t* dims, int n, int64_t* str) {
  int64_t s = 1;
  for (int i = 0; i < n; ++i) {
    str[i] = s;
    s *= dims[i];
  }
}

// ------------------------------------------------------------------------------------------
// Copy tasks
// ------------------------------------------------------------------------------------------
void CopyTask::simplify() {
  int m = 0;
  for (int i = 0; i < nd; ++i) {
    if (ext[i] == 1) continue;
    ext[m] = ext[i];
    sstr[m] = sstr[i];
    dstr[m] = dstr[i];
    ++m;
  }
  nd = m;
  // merge axis i+1 into i when it continues i contiguously in both src and dst
  int k = 0;
  for (int i = 0; i < nd; ++i) {
    if (k > 0 && sstr[i] == sstr[k - 1] * ext[k - 1] && dstr[i] == dstr[k - 1] * ext[k - 1]) {
      ext[k - 1] *= ext[i];
      continue;
    }
    ext[k] = ext[i];
    sstr[k] = sstr[i];
    dstr[k] = dstr[i];
    ++k;
  }
  nd = k;
  if (nd == 0) {  // a single element
    nd = 1;
    ext[0] = 1;
    sstr[0] = 1;
    dstr[0] = 1;
  }
}

static bool tasks_identity(const std::vector<CopyTask>& tasks, int64_t total) {
  // identity when every task copies a contiguous range onto the same range
  int64_t covered = 0;
  for (auto& t : tasks) {
    if (t.soff != t.doff) return false;
    if (!(t.nd == 1 && t.sstr[0] == 1 && t.dstr[0] == 1)) return false;
    covered += t.numel();
  }
  return covered == total;
}

// ------------------------------------------------------------------------------------------
// permutelegs (symreleg.jl:34-51)
// ------------------------------------------------------------------------------------------
static void check_perm(const std::vector<int>& perm1, int N) {
  std::vector<int> s = perm1;
  std::sort(s.begin(), s.end());
  for (int i = 0; i < N; ++i)
    if ((int)s.size() != N || s[i] != i + 1) fail(kErrArgument, "Not a valid permutation!");
}

RelegPlan plan_permutelegs(const TensorMeta& A, const std::vector<int>& perm1) {
  const int N = A.N();
  check_perm(perm1, N);
  RelegPlan P;
  std::vector<Space> sp(N);
  for (int i = 0; i < N; ++i) sp[i] = A.space[perm1[i] - 1];
  P.out = TensorMeta::build(A.charge, sp);
  if (P.out.nblocks() != A.nblocks()) fail(kErrSpaceMismatch, "permutelegs: sector count");
  int lab[kMaxLegs];
  for (size_t b = 0; b < A.nblocks(); ++b) {
    const int* s = A.sec.labels(b);
    const int64_t* z = A.sec.sizes(b);
    for (int i = 0; i < N; ++i) lab[i] = s[perm1[i] - 1];
    long ob = P.out.find(lab);
    if (ob < 0) fail(kErrSpaceMismatch, "permutelegs: missing sector");
    int64_t sstr[kMaxLegs], ostr[kMaxLegs], odims[kMaxLegs];
    colmajor_strides(z, N, sstr);
    for (int i = 0; i < N; ++i) odims[i] = z[perm1[i] - 1];
    colmajor_strides(odims, N, ostr);
    CopyTask t;
    t.nd = N;
    for (int j = 0; j < N; ++j) {  // iterate in source axis order
      t.ext[j] = z[j];
      t.sstr[j] = sstr[j];
    }
    for (int i = 0; i < N; ++i) t.dstr[perm1[i] - 1] = ostr[i];
    t.soff = A.off[b];
    t.doff = P.out.off[ob];
    t.simplify();
    P.tasks.push_back(t);
  }
  P.identity = tasks_identity(P.tasks, A.total);
  return P;
}

// ------------------------------------------------------------------------------------------
// fuselegs (symreleg.jl:79-146)
// ------------------------------------------------------------------------------------------
RelegPlan plan_fuselegs(const TensorMeta& A, int l1, int n, bool dual) {
  const int N = A.N();
  if (!(0 < l1 && l1 < N + 2 - n) || n < 1)
    fail(kErrArgument, "fuselegs " + std::to_string(l1) + " to " + std::to_string(l1 + n - 1) +
                           " for size " + std::to_string(N));
  const int i0 = l1 - 1, i1 = l1 - 1 + n;
  RelegPlan P;
  if (n < 2 && dual == A.space[i0].dual) {
    P.out = A;
    P.identity = true;
    CopyTask t;
    t.nd = 1;
    t.ext[0] = A.total;
    t.sstr[0] = t.dstr[0] = 1;
    if (A.total) P.tasks.push_back(t);
    return P;
  }
  const int Nf = N - n + 1;
  std::vector<int> fs(A.nblocks() * Nf);
  for (size_t b = 0; b < A.nblocks(); ++b) {
    const int* s = A.sec.labels(b);
    int fc = 0;
    for (int k = i0; k < i1; ++k) fc += eff(s[k], A.space[k].dual);
    if (dual) fc = -fc;
    int* f = fs.data() + b * Nf;
    int q = 0;
    for (int k = 0; k < i0; ++k) f[q++] = s[k];
    f[q++] = fc;
    for (int k = i1; k < N; ++k) f[q++] = s[k];
  }
  auto sperm = stable_sortperm(fs, Nf);
  std::vector<Space> sub(A.space.begin() + i0, A.space.begin() + i1);
  std::vector<Space> sp(A.space.begin(), A.space.begin() + i0);
  sp.push_back(fuse(dual, sub));
  sp.insert(sp.end(), A.space.begin() + i1, A.space.end());
  P.out = TensorMeta::build(A.charge, sp);
  size_t ptr = 0;
  for (size_t ob = 0; ob < P.out.nblocks(); ++ob) {
    const int64_t* z = P.out.sec.sizes(ob);
    int64_t ostr[kMaxLegs];
    colmajor_strides(z, Nf, ostr);
    int64_t p = 0;
    while (p < z[i0]) {
      if (ptr >= sperm.size()) fail(kErrSpaceMismatch, "fuselegs: source blocks exhausted");
      size_t b = sperm[ptr];
      const int64_t* s = A.sec.sizes(b);
      int64_t fd = 1;
      for (int k = i0; k < i1; ++k) fd *= s[k];
      CopyTask t;
      t.nd = N;
      int64_t sstr[kMaxLegs];
      colmajor_strides(s, N, sstr);
      int64_t inner = 1;
      for (int k = 0; k < N; ++k) {
        t.ext[k] = s[k];
        t.sstr[k] = sstr[k];
        if (k < i0) t.dstr[k] = ostr[k];
        else if (k < i1) {
          t.dstr[k] = ostr[i0] * inner;
          inner *= s[k];
        } else t.dstr[k] = ostr[k - n + 1];
      }
      t.soff = A.off[b];
      t.doff = P.out.off[ob] + p * ostr[i0];
      t.simplify();
      P.tasks.push_back(t);
      p += fd;
      ++ptr;
    }
    if (p != z[i0]) fail(kErrSpaceMismatch, "fuselegs: fused block size mismatch");
  }
  if (ptr != A.nblocks()) fail(kErrSpaceMismatch, "fuselegs: unused source blocks");
  P.identity = tasks_identity(P.tasks, A.total);
  return P;
}

// ------------------------------------------------------------------------------------------
// splitleg (symreleg.jl:160-214)
// ------------------------------------------------------------------------------------------
RelegPlan plan_splitleg(const TensorMeta& A, int l1, const std::vector<Space>& sp) {
  const int N = A.N();
  if (!(0 < l1 && l1 <= N)) fail(kErrArgument, "integer l not in range");
  const int i = l1 - 1;
  const int M = (int)sp.size();
  RelegPlan P;
  if (M == 1) {
    if (A.space[i] != sp[0]) fail(kErrSpaceMismatch, "SpaceMismatch in splitleg");
    P.out = A;
    P.identity = true;
    CopyTask t;
    t.nd = 1;
    t.ext[0] = A.total;
    t.sstr[0] = t.dstr[0] = 1;
    if (A.total) P.tasks.push_back(t);
    return P;
  }
  const int No = N + M - 1;
  if (No > kMaxLegs) fail(kErrArgument, "too many legs");
  std::vector<Space> nsp(A.space.begin(), A.space.begin() + i);
  nsp.insert(nsp.end(), sp.begin(), sp.end());
  nsp.insert(nsp.end(), A.space.begin() + i + 1, A.space.end());
  P.out = TensorMeta::build(A.charge, nsp);
  std::vector<size_t> order(A.nblocks());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t a, size_t b) { return A.sec.labels(a)[i] < A.sec.labels(b)[i]; });
  size_t produced = 0;
  for (size_t b : order) {
    const int* s = A.sec.labels(b);
    const int64_t* z = A.sec.sizes(b);
    int charge = eff(s[i], A.space[i].dual);
    SectorList pats = allsectorsandsizes(charge, sp);
    int64_t sstr[kMaxLegs];
    colmajor_strides(z, N, sstr);
    int64_t pivot = 0;
    for (size_t pi = 0; pi < pats.count(); ++pi) {
      int lab[kMaxLegs];
      int64_t dz[kMaxLegs];
      int q = 0;
      for (int k = 0; k < i; ++k) { lab[q] = s[k]; dz[q++] = z[k]; }
      for (int k = 0; k < M; ++k) { lab[q] = pats.labels(pi)[k]; dz[q++] = pats.sizes(pi)[k]; }
      for (int k = i + 1; k < N; ++k) { lab[q] = s[k]; dz[q++] = z[k]; }
      long ob = P.out.find(lab);
      if (ob < 0) fail(kErrSpaceMismatch, "splitleg: sector not allowed");
      int64_t sl = pats.numel(pi);
      if (pivot + sl > z[i]) fail(kErrSpaceMismatch, "splitleg: leg sizes do not match");
      CopyTask t;
      t.nd = No;
      int64_t dstr[kMaxLegs];
      colmajor_strides(dz, No, dstr);
      int64_t inner = 1;
      for (int k = 0; k < No; ++k) {
        t.ext[k] = dz[k];
        t.dstr[k] = dstr[k];
        if (k < i) t.sstr[k] = sstr[k];
        else if (k < i + M) {
          t.sstr[k] = sstr[i] * inner;
          inner *= dz[k];
        } else t.sstr[k] = sstr[k - M + 1];
      }
      t.soff = A.off[b] + pivot * sstr[i];
      t.doff = P.out.off[ob];
      t.simplify();
      P.tasks.push_back(t);
      pivot += sl;
      ++produced;
    }
    if (pivot != z[i]) fail(kErrSpaceMismatch, "splitleg: leg sizes do not match");
  }
  if (produced != P.out.nblocks()) fail(kErrSpaceMismatch, "splitleg: sectors not covered");
  P.identity = tasks_identity(P.tasks, A.total);
  return P;
}

// ------------------------------------------------------------------------------------------
// SymMatrix (contract.jl:112-171)
// ------------------------------------------------------------------------------------------
FusePlan plan_symmatrix(const TensorMeta& A, const std::vector<int>& rows1,
                        const std::vector<int>& cols1) {
  return plan_symmatrix_rec(A, rows1, cols1, nullptr);
}

FusePlan plan_symmatrix_rec(const TensorMeta& A, const std::vector<int>& rows1,
                            const std::vector<int>& cols1, std::vector<BlockMap>* rec) {
  const int N = A.N();
  if (rec) rec->assign(A.nblocks(), BlockMap());
  std::vector<int> idxperm = rows1;
  idxperm.insert(idxperm.end(), cols1.begin(), cols1.end());
  {
    std::vector<int> s = idxperm;
    std::sort(s.begin(), s.end());
    bool ok = (int)s.size() == N;
    for (int i = 0; ok && i < N; ++i) ok = s[i] == i + 1;
    if (!ok) fail(kErrArgument, "Incorrect index set for conversion to SymMatrix!");
  }
  if (rows1.empty()) fail(kErrArgument, "empty row for matrix not allowed!");
  if (cols1.empty()) fail(kErrArgument, "empty col for matrix not allowed!");
  const int n = (int)rows1.size();
  const size_t nb = A.nblocks();
  std::vector<int> csects(nb * N);
  for (size_t b = 0; b < nb; ++b)
    for (int k = 0; k < N; ++k) csects[b * N + k] = A.sec.labels(b)[idxperm[k] - 1];
  auto sperm1 = stable_sortperm(csects, N);
  std::vector<int> fsects(nb * 2);
  for (size_t j = 0; j < nb; ++j) {
    const int* sec = csects.data() + sperm1[j] * N;
    int c1 = 0, c2 = 0;
    for (int k = 0; k < n; ++k) c1 += eff(sec[k], A.space[rows1[k] - 1].dual);
    for (int k = n; k < N; ++k) c2 += eff(sec[k], A.space[cols1[k - n] - 1].dual);
    fsects[2 * j] = c1;
    fsects[2 * j + 1] = -c2;
  }
  auto sperm2 = stable_sortperm(fsects, 2);
  std::vector<size_t> semits(nb);
  for (size_t j = 0; j < nb; ++j) semits[j] = sperm1[sperm2[j]];

  std::vector<Space> rs, cs;
  for (int r : rows1) rs.push_back(A.space[r - 1]);
  for (int c : cols1) cs.push_back(A.space[c - 1]);
  FusePlan P;
  P.out = TensorMeta::build(A.charge, {fuse(false, rs), fuse(true, cs)});
  size_t ptr = 0;
  for (size_t f = 0; f < P.out.nblocks(); ++f) {
    const int64_t rlim = P.out.sec.sizes(f)[0], clim = P.out.sec.sizes(f)[1];
    int64_t pc = 0;
    while (pc < clim) {
      int64_t pr = 0, fdc = 0;
      while (pr < rlim) {
        if (ptr >= nb) fail(kErrSpaceMismatch, "SymMatrix: source blocks exhausted");
        size_t b = semits[ptr];
        const int64_t* z = A.sec.sizes(b);
        int64_t sstr[kMaxLegs];
        colmajor_strides(z, N, sstr);
        CopyTask t;
        t.nd = N;
        int64_t fdr = 1;
        fdc = 1;
        for (int k = 0; k < N; ++k) {
          int leg = idxperm[k] - 1;
          t.ext[k] = z[leg];
          t.sstr[k] = sstr[leg];
          if (k < n) {
            t.dstr[k] = fdr;
            fdr *= z[leg];
          } else {
            t.dstr[k] = rlim * fdc;
            fdc *= z[leg];
          }
        }
        t.soff = A.off[b];
        t.doff = P.out.off[f] + pr + pc * rlim;
        if (rec) {  // destination of source block b in its natural axis order
          BlockMap& m = (*rec)[b];
          m.off = t.doff;
          for (int k = 0; k < N; ++k) m.str[idxperm[k] - 1] = t.dstr[k];
        }
        t.simplify();
        P.tasks.push_back(t);
        pr += fdr;
        ++ptr;
      }
      if (pr != rlim) fail(kErrSpaceMismatch, "SymMatrix: row sizes do not tile");
      pc += fdc;
    }
    if (pc != clim) fail(kErrSpaceMismatch, "SymMatrix: column sizes do not tile");
  }
  if (ptr != nb) fail(kErrSpaceMismatch, "SymMatrix: unused source blocks");
  P.identity = tasks_identity(P.tasks, A.total);
  return P;
}

// ------------------------------------------------------------------------------------------
// Block GEMM (contract.jl:234-298)
// ------------------------------------------------------------------------------------------
MatmulPlan plan_matmul(const TensorMeta& A, const TensorMeta& B) {
  if (A.N() != 2 || B.N() != 2) fail(kErrArgument, "matmul needs rank-2 tensors");
  if (!isdual_pair(A.space[1], B.space[0])) fail(kErrSpaceMismatch, "not contractible!");
  MatmulPlan P;
  P.out = TensorMeta::build(A.charge + B.charge, {A.space[0], B.space[1]});
  for (size_t i = 0; i < P.out.nblocks(); ++i) {
    const int c1 = P.out.sec.labels(i)[0], c2 = P.out.sec.labels(i)[1];
    const int _c1 = eff(c1, A.space[0].dual), _c2 = eff(c2, B.space[1].dual);
    int sa[2], sb[2];
    sa[0] = c1;
    sb[1] = c2;
    if (A.space[1].dual) {
      sa[1] = -A.charge + _c1;
      sb[0] = B.charge - _c2;
    } else {
      sa[1] = A.charge - _c1;
      sb[0] = -B.charge + _c2;
    }
    long ia = A.find(sa), ib = B.find(sb);
    GemmTask g;
    g.M = P.out.sec.sizes(i)[0];
    g.N = P.out.sec.sizes(i)[1];
    g.offC = P.out.off[i];
    g.ldc = g.M;
    if (ia >= 0 && ib >= 0) {
      g.K = A.sec.sizes(ia)[1];
      if (B.sec.sizes(ib)[0] != g.K) fail(kErrSpaceMismatch, "matmul: inner sizes differ");
      g.offA = A.off[ia];
      g.offB = B.off[ib];
      g.lda = g.M;
      g.ldb = g.K;
      P.flops += 2.0 * g.M * g.N * g.K;
    } else {
      g.K = 0;
      g.offA = g.offB = 0;
      g.lda = g.ldb = 1;
    }
    P.gemms.push_back(g);
  }
  return P;
}

// ------------------------------------------------------------------------------------------
// SymTensor(::SymMatrix, rlegs, clegs) + permutelegs (contract.jl:187-224, 45-46)
// ------------------------------------------------------------------------------------------
RelegPlan plan_split_permute(const TensorMeta& C, const std::vector<Space>& rlegs,
                             const std::vector<Space>& clegs, const std::vector<int>& perm1) {
  return plan_split_permute_rec(C, rlegs, clegs, perm1, nullptr);
}

RelegPlan plan_split_permute_rec(const TensorMeta& C, const std::vector<Space>& rlegs,
                                 const std::vector<Space>& clegs, const std::vector<int>& perm1,
                                 std::vector<BlockMap>* rec) {
  const int nr = (int)rlegs.size(), nc = (int)clegs.size(), N = nr + nc;
  if (N > kMaxLegs) fail(kErrArgument, "too many legs");
  check_perm(perm1, N);
  std::vector<Space> inter(rlegs);
  inter.insert(inter.end(), clegs.begin(), clegs.end());
  std::vector<Space> fsp(N);
  for (int i = 0; i < N; ++i) fsp[i] = inter[perm1[i] - 1];
  RelegPlan P;
  P.out = TensorMeta::build(C.charge, fsp);
  if (rec) rec->assign(P.out.nblocks(), BlockMap());
  size_t produced = 0;
  for (size_t b = 0; b < C.nblocks(); ++b) {
    int c1 = eff(C.sec.labels(b)[0], C.space[0].dual);
    int c2 = eff(C.sec.labels(b)[1], C.space[1].dual);
    const int64_t ld = C.sec.sizes(b)[0];
    SectorList rp = allsectorsandsizes(c1, rlegs), cp = allsectorsandsizes(c2, clegs);
    int64_t pc = 0;
    for (size_t j = 0; j < cp.count(); ++j) {
      int64_t csl = cp.numel(j), pr = 0;
      for (size_t i = 0; i < rp.count(); ++i) {
        int64_t rsl = rp.numel(i);
        int lab[kMaxLegs], flab[kMaxLegs];
        int64_t dz[kMaxLegs], fdz[kMaxLegs], sstr[kMaxLegs], fstr[kMaxLegs];
        int64_t s = 1;
        for (int k = 0; k < nr; ++k) {
          lab[k] = rp.labels(i)[k];
          dz[k] = rp.sizes(i)[k];
          sstr[k] = s;
          s *= dz[k];
        }
        s = ld;
        for (int k = 0; k < nc; ++k) {
          lab[nr + k] = cp.labels(j)[k];
          dz[nr + k] = cp.sizes(j)[k];
          sstr[nr + k] = s;
          s *= dz[nr + k];
        }
        for (int k = 0; k < N; ++k) {
          flab[k] = lab[perm1[k] - 1];
          fdz[k] = dz[perm1[k] - 1];
        }
        colmajor_strides(fdz, N, fstr);
        long ob = P.out.find(flab);
        if (ob < 0) fail(kErrSpaceMismatch, "split: sector not allowed");
        CopyTask t;
        t.nd = N;
        for (int k = 0; k < N; ++k) {
          t.ext[k] = dz[k];
          t.sstr[k] = sstr[k];
        }
        for (int k = 0; k < N; ++k) t.dstr[perm1[k] - 1] = fstr[k];
        t.soff = C.off[b] + pr + pc * ld;
        t.doff = P.out.off[ob];
        if (rec) {  // source of output block ob in its natural axis order
          BlockMap& m = (*rec)[ob];
          m.off = t.soff;
          for (int k = 0; k < N; ++k) m.str[k] = sstr[perm1[k] - 1];
        }
        t.simplify();
        P.tasks.push_back(t);
        ++produced;
        pr += rsl;
      }
      if (pr != ld) fail(kErrSpaceMismatch, "split: row sizes do not tile");
      pc += csl;
    }
    if (pc != C.sec.sizes(b)[1]) fail(kErrSpaceMismatch, "split: column sizes do not tile");
  }
  if (produced != P.out.nblocks()) fail(kErrSpaceMismatch, "split: sectors not covered");
  P.identity = tasks_identity(P.tasks, C.total);
  return P;
}

std::vector<CopyTask> compose_through(const TensorMeta& X, const std::vector<BlockMap>& src_of_x,
                                      const std::vector<BlockMap>& dst_of_x) {
  if (src_of_x.size() != X.nblocks() || dst_of_x.size() != X.nblocks())
    fail(kErrArgument, "compose_through: block maps do not match the intermediate");
  std::vector<CopyTask> out;
  out.reserve(X.nblocks());
  const int N = X.N();
  for (size_t b = 0; b < X.nblocks(); ++b) {
    CopyTask t;
    t.nd = N;
    for (int k = 0; k < N; ++k) {
      t.ext[k] = X.sec.sizes(b)[k];
      t.sstr[k] = src_of_x[b].str[k];
      t.dstr[k] = dst_of_x[b].str[k];
    }
    t.soff = src_of_x[b].off;
    t.doff = dst_of_x[b].off;
    t.simplify();
    out.push_back(t);
  }
  return out;
}

// ------------------------------------------------------------------------------------------
// contract (contract.jl:11-47, 82-99)
// ------------------------------------------------------------------------------------------
void contract_index_perm(const std::vector<int>& idx, std::vector<int>& rems,
                         std::vector<int>& cons, std::vector<int>& tofinals) {
  std::vector<int> r, c, corder, tof;
  for (size_t i = 0; i < idx.size(); ++i) {
    if (idx[i] < 0) {
      c.push_back((int)i + 1);
      corder.push_back(idx[i]);
    } else {
      r.push_back((int)i + 1);
      tof.push_back(idx[i]);
    }
  }
  std::vector<size_t> p(tof.size()), q(corder.size());
  std::iota(p.begin(), p.end(), 0);
  std::iota(q.begin(), q.end(), 0);
  std::stable_sort(p.begin(), p.end(), [&](size_t a, size_t b) { return tof[a] < tof[b]; });
  std::stable_sort(q.begin(), q.end(),
                   [&](size_t a, size_t b) { return std::abs(corder[a]) < std::abs(corder[b]); });
  rems.clear();
  cons.clear();
  tofinals.clear();
  for (size_t k : p) {
    rems.push_back(r[k]);
    tofinals.push_back(tof[k]);
  }
  for (size_t k : q) cons.push_back(c[k]);
}

std::shared_ptr<ContractPlan> plan_contract(const TensorMeta& A, const std::vector<int>& idxA,
                                            const TensorMeta& B, const std::vector<int>& idxB) {
  if ((int)idxA.size() != A.N() || (int)idxB.size() != B.N())
    fail(kErrArgument, "index tuple length differs from tensor rank");
  std::vector<int> remsA, consA, tofA, remsB, consB, tofB;
  contract_index_perm(idxA, remsA, consA, tofA);
  contract_index_perm(idxB, remsB, consB, tofB);
  auto P = std::make_shared<ContractPlan>();
  if (remsA.empty() || remsB.empty()) {
    if (!(remsA.empty() && remsB.empty()))
      fail(kErrUnsupported,
           "contract with no remaining leg on one operand only is undefined in the reference");
    // both fully contracted: SymVector(A) * SymVector(B) (contract.jl:24-28, 226-232)
    P->scalar = true;
    P->fa.out = plan_fuselegs(plan_permutelegs(A, consA).out, 1, A.N(), false).out;
    P->fb.out = plan_fuselegs(plan_permutelegs(B, consB).out, 1, B.N(), true).out;
    if (!isdual_pair(P->fa.out.space[0], P->fb.out.space[0]))
      fail(kErrSpaceMismatch, "not contractible!");
    return P;
  }
  P->fa = plan_symmatrix(A, remsA, consA);
  P->fb = plan_symmatrix(B, consB, remsB);
  P->rowsA = remsA;
  P->colsA = consA;
  P->rowsB = consB;
  P->colsB = remsB;
  P->mm = plan_matmul(P->fa.out, P->fb.out);
  std::vector<Space> rl, cl;
  for (int r : remsA) rl.push_back(A.space[r - 1]);
  for (int r : remsB) cl.push_back(B.space[r - 1]);
  std::vector<int> fin = tofA;
  fin.insert(fin.end(), tofB.begin(), tofB.end());
  std::vector<int> inv(fin.size());
  for (size_t i = 0; i < fin.size(); ++i) {
    if (fin[i] < 1 || fin[i] > (int)fin.size()) fail(kErrArgument, "bad output label");
    inv[fin[i] - 1] = (int)i + 1;
  }
  P->split = plan_split_permute(P->mm.out, rl, cl, inv);
  P->flops = P->mm.flops;
  P->rlegs = rl;
  P->clegs = cl;
  P->perm = inv;
  return P;
}

static void apply_tasks_host(const std::vector<CopyTask>& tasks, const std::vector<int64_t>& src,
                             std::vector<int64_t>& dst) {
  for (const CopyTask& t : tasks) {
    int64_t idx[kMaxTaskDims] = {0};
    int64_t s = t.soff, d = t.doff;
    for (;;) {
      dst[d] = src[s];
      int i = 0;
      for (; i < t.nd; ++i) {
        if (++idx[i] < t.ext[i]) {
          s += t.sstr[i];
          d += t.dstr[i];
          break;
        }
        s -= (t.ext[i] - 1) * t.sstr[i];
        d -= (t.ext[i] - 1) * t.dstr[i];
        idx[i] = 0;
      }
      if (i == t.nd) break;
    }
  }
}

void check_composition(const std::vector<CopyTask>& step1, int64_t n_src, int64_t n_mid,
                       const std::vector<CopyTask>& step2, int64_t n_dst,
                       const std::vector<CopyTask>& composed) {
  validate_copy_tasks(step1, n_src, n_mid);
  validate_copy_tasks(step2, n_mid, n_dst);
  validate_copy_tasks(composed, n_src, n_dst);
  std::vector<int64_t> src(n_src), mid(n_mid, -1), a(n_dst, -1), b(n_dst, -2);
  for (int64_t i = 0; i < n_src; ++i) src[i] = i;
  apply_tasks_host(step1, src, mid);
  apply_tasks_host(step2, mid, a);
  apply_tasks_host(composed, src, b);
  if (a != b) fail(kErrArgument, "composed copy plan differs from the two-step plan");
}

// ------------------------------------------------------------------------------------------
// self-checks
// ------------------------------------------------------------------------------------------
void validate_copy_tasks(const std::vector<CopyTask>& tasks, int64_t src_total,
                         int64_t dst_total) {
  std::vector<uint8_t> hit(dst_total, 0);
  for (size_t k = 0; k < tasks.size(); ++k) {
    const CopyTask& t = tasks[k];
    if (t.nd < 1 || t.nd > kMaxTaskDims) fail(kErrArgument, "task rank out of range");
    int64_t smin = t.soff, smax = t.soff, dmin = t.doff, dmax = t.doff;
    for (int i = 0; i < t.nd; ++i) {
      if (t.ext[i] < 1) fail(kErrArgument, "task extent < 1");
      smax += (t.ext[i] - 1) * t.sstr[i];
      dmax += (t.ext[i] - 1) * t.dstr[i];
      if (t.sstr[i] < 0 || t.dstr[i] < 0) fail(kErrArgument, "negative stride");
    }
    if (smin < 0 || smax >= src_total || dmin < 0 || dmax >= dst_total)
      fail(kErrArgument, "copy task " + std::to_string(k) + " out of bounds");
    // walk every element (odometer) and mark its destination
    int64_t idx[kMaxTaskDims] = {0};
    int64_t d = t.doff;
    for (;;) {
      if (hit[d]) fail(kErrArgument, "destination element written twice");
      hit[d] = 1;
      int i = 0;
      for (; i < t.nd; ++i) {
        if (++idx[i] < t.ext[i]) {
          d += t.dstr[i];
          break;
        }
        d -= (t.ext[i] - 1) * t.dstr[i];
        idx[i] = 0;
      }
      if (i == t.nd) break;
    }
  }
  for (int64_t i = 0; i < dst_total; ++i)
    if (!hit[i]) fail(kErrArgument, "destination element never written");
}

void validate_gemms(const std::vector<GemmTask>& gs, int64_t a_total, int64_t b_total,
                    int64_t c_total) {
  std::vector<uint8_t> hit(c_total, 0);
  for (const GemmTask& g : gs) {
    if (g.M < 1 || g.N < 1 || g.K < 0) fail(kErrArgument, "GEMM with empty M or N");
    if (g.ldc < g.M || g.offC < 0 || g.offC + (g.M - 1) + (g.N - 1) * g.ldc >= c_total)
      fail(kErrArgument, "GEMM C window out of bounds");
    if (g.K > 0) {
      if (g.lda < g.M || g.offA < 0 || g.offA + (g.M - 1) + (g.K - 1) * g.lda >= a_total)
        fail(kErrArgument, "GEMM A window out of bounds");
      if (g.ldb < g.K || g.offB < 0 || g.offB + (g.K - 1) + (g.N - 1) * g.ldb >= b_total)
        fail(kErrArgument, "GEMM B window out of bounds");
    }
    for (int64_t n = 0; n < g.N; ++n)
      for (int64_t m = 0; m < g.M; ++m) {
        int64_t c = g.offC + m + n * g.ldc;
        if (hit[c]) fail(kErrArgument, "GEMM output written twice");
        hit[c] = 1;
      }
  }
  for (int64_t i = 0; i < c_total; ++i)
    if (!hit[i]) fail(kErrArgument, "GEMM output element never written");
}

void validate_contract(const ContractPlan& p, const TensorMeta& A, const TensorMeta& B) {
  if (p.scalar) return;
  validate_copy_tasks(p.fa.tasks, A.total, p.fa.out.total);
  validate_copy_tasks(p.fb.tasks, B.total, p.fb.out.total);
  validate_gemms(p.mm.gemms, p.fa.out.total, p.fb.out.total, p.mm.out.total);
  validate_copy_tasks(p.split.tasks, p.mm.out.total, p.split.out.total);
}

}  // namespace mpsg
