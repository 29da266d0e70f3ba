// Host-side symbolic set-up (see cxg_plan.h).
#include "cxg_plan.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <utility>

namespace cxg {

static std::string checkCsc(const char* name, int rows, int cols, const int* p, const int* i) {
  if (!p || (!i && p[cols] > 0)) return std::string(name) + ": null index array";
  if (p[0] != 0) return std::string(name) + ": column pointer must start at 0";
  for (int c = 0; c < cols; ++c) {
    if (p[c + 1] < p[c]) return std::string(name) + ": column pointers must be non-decreasing";
    for (int k = p[c]; k < p[c + 1]; ++k) {
      if (i[k] < 0 || i[k] >= rows) return std::string(name) + ": row index out of range";
      if (k > p[c] && i[k] <= i[k - 1])
        return std::string(name) + ": row indices must be strictly increasing within a column";
    }
  }
  return "";
}

std::string validateProblem(const cxg_problem& pr) {
  if (pr.zero_dim < 0 || pr.nonneg_dim < 0 || pr.n_soc < 0) return "invalid cone spec (negative dimension)";
  int64_t m = (int64_t)pr.zero_dim + pr.nonneg_dim;
  for (int k = 0; k < pr.n_soc; ++k) {
    if (!pr.soc_dims || pr.soc_dims[k] < 1) return "invalid cone spec (SOC dimension < 1)";
    m += pr.soc_dims[k];
  }
  if (pr.n < 1) return "n must be >= 1";
  if (m != pr.m) return "A rows / b size do not match the cone spec's total dimension";
  if (m > (1 << 28) || pr.n > (1 << 28)) return "instance too large";
  if (!pr.q || (pr.m > 0 && !pr.b)) return "null q or b";
  std::string e = checkCsc("P", pr.n, pr.n, pr.Pp, pr.Pi);
  if (!e.empty()) return e;
  e = checkCsc("A", pr.m, pr.n, pr.Ap, pr.Ai);
  if (!e.empty()) return e;
  if (pr.Pp[pr.n] > 0 && !pr.Px) return "null P values";
  if (pr.Ap[pr.n] > 0 && !pr.Ax) return "null A values";
  return "";
}

void computeEquilibration(const cxg_problem& pr, const cxg_settings& st, std::vector<double>& d,
                          std::vector<double>& e, double& c) {
  const int n = pr.n, m = pr.m;
  d.assign((size_t)n, 1.0);
  e.assign((size_t)m, 1.0);
  c = 1.0;
  if (!st.equilibrate || n == 0) return;
  const int nnzP = pr.Pp[n], nnzA = pr.Ap[n];
  std::vector<double> Pw(pr.Px, pr.Px + nnzP), Aw(pr.Ax, pr.Ax + nnzA);
  std::vector<double> nx((size_t)n), nz((size_t)m), dx((size_t)n), dz((size_t)m);
  const double minS = st.equilibrate_min_scale, maxS = st.equilibrate_max_scale;
  const int socBase = pr.zero_dim + pr.nonneg_dim;
  for (int it = 0; it < st.equilibrate_max_iter; ++it) {
    std::fill(nx.begin(), nx.end(), 0.0);
    std::fill(nz.begin(), nz.end(), 0.0);
    for (int col = 0; col < n; ++col)
      for (int k = pr.Pp[col]; k < pr.Pp[col + 1]; ++k) {
        const double av = std::abs(Pw[(size_t)k]);
        const int r = pr.Pi[k];
        nx[(size_t)r] = std::max(nx[(size_t)r], av);
        nx[(size_t)col] = std::max(nx[(size_t)col], av);
      }
    for (int col = 0; col < n; ++col)
      for (int k = pr.Ap[col]; k < pr.Ap[col + 1]; ++k) {
        const double av = std::abs(Aw[(size_t)k]);
        nx[(size_t)col] = std::max(nx[(size_t)col], av);
        nz[(size_t)pr.Ai[k]] = std::max(nz[(size_t)pr.Ai[k]], av);
      }
    // one shared value per SOC block (equilibration.cpp:50-57)
    int off = socBase;
    for (int b = 0; b < pr.n_soc; ++b) {
      const int dim = pr.soc_dims[b];
      double mx = nz[(size_t)off];
      for (int t = 1; t < dim; ++t) mx = std::max(mx, nz[(size_t)(off + t)]);
      for (int t = 0; t < dim; ++t) nz[(size_t)(off + t)] = mx;
      off += dim;
    }
    for (int t = 0; t < n; ++t) dx[(size_t)t] = 1.0 / std::sqrt(nx[(size_t)t] > 0 ? nx[(size_t)t] : 1.0);
    for (int t = 0; t < m; ++t) dz[(size_t)t] = 1.0 / std::sqrt(nz[(size_t)t] > 0 ? nz[(size_t)t] : 1.0);
    for (int col = 0; col < n; ++col)
      for (int k = pr.Pp[col]; k < pr.Pp[col + 1]; ++k) Pw[(size_t)k] *= dx[(size_t)pr.Pi[k]] * dx[(size_t)col];
    for (int col = 0; col < n; ++col)
      for (int k = pr.Ap[col]; k < pr.Ap[col + 1]; ++k) Aw[(size_t)k] *= dz[(size_t)pr.Ai[k]] * dx[(size_t)col];
    for (int t = 0; t < n; ++t) d[(size_t)t] *= dx[(size_t)t];
    for (int t = 0; t < m; ++t) e[(size_t)t] *= dz[(size_t)t];
  }
  for (double& v : d) v = std::min(std::max(v, minS), maxS);
  for (double& v : e) v = std::min(std::max(v, minS), maxS);
  double sumAbs = 0.0;
  for (int k = 0; k < nnzP; ++k) sumAbs += std::abs(Pw[(size_t)k]);
  if (nnzP > 0) {
    const double meanAbs = sumAbs / (double)nnzP;
    if (meanAbs > 0) c = 1.0 / std::max(meanAbs, minS);
  }
  c = std::min(std::max(c, minS), maxS);
}

bool samePattern(const std::vector<int>& p_ref, const std::vector<int>& i_ref, int cols,
                 const int* p, const int* i) {
  if ((int)p_ref.size() != cols + 1) return false;
  if (!std::equal(p, p + cols + 1, p_ref.begin())) return false;
  const int nz = p[cols];
  if ((int)i_ref.size() != nz) return false;
  return nz == 0 || std::equal(i, i + nz, i_ref.begin());
}

std::string checkPlanCounts(const cxg_problem& pr) {
  const int n = pr.n, m = pr.m, p = pr.zero_dim, l = pr.nonneg_dim;
  int64_t upperOff = 0, diag = 0;
  for (int c = 0; c < n; ++c)
    for (int k = pr.Pp[c]; k < pr.Pp[c + 1]; ++k) {
      if (pr.Pi[k] < c) ++upperOff;
      else if (pr.Pi[k] == c) ++diag;
    }
  const int64_t nnzPs = 2 * upperOff + diag;
  // A's rows: count entries per row, then each unit's distinct columns with a stamp per column
  std::vector<int> rowStart((size_t)m + 1, 0);
  for (int k = 0; k < pr.Ap[n]; ++k) rowStart[(size_t)pr.Ai[k] + 1]++;
  for (int r = 0; r < m; ++r) rowStart[(size_t)r + 1] += rowStart[(size_t)r];
  std::vector<int> rowCols((size_t)pr.Ap[n]);
  {
    std::vector<int> fill(rowStart.begin(), rowStart.end() - 1);
    for (int c = 0; c < n; ++c)
      for (int k = pr.Ap[c]; k < pr.Ap[c + 1]; ++k) rowCols[(size_t)fill[(size_t)pr.Ai[k]]++] = c;
  }
  std::vector<int> stamp((size_t)n, -1);
  int64_t nAd = 0, nContrib = 0;
  int r0 = p + l;
  const int nUnits = l + pr.n_soc;
  for (int u = 0; u < nUnits; ++u) {
    const int lo = (u < l) ? p + u : r0;
    const int d = (u < l) ? 1 : pr.soc_dims[u - l];
    if (u >= l) r0 += d;
    int64_t s = 0;
    for (int r = lo; r < lo + d; ++r)
      for (int k = rowStart[(size_t)r]; k < rowStart[(size_t)r + 1]; ++k)
        if (stamp[(size_t)rowCols[(size_t)k]] != u) { stamp[(size_t)rowCols[(size_t)k]] = u; ++s; }
    nAd += (int64_t)d * s;
    nContrib += s * (s + 1) / 2;
  }
  if (nnzPs > INT32_MAX)
    return "the full symmetric P has " + std::to_string(nnzPs) + " entries, above the plan's 32-bit limit " +
           std::to_string(INT32_MAX);
  if (nAd > INT32_MAX)
    return "the densified cone-unit A blocks hold " + std::to_string(nAd) + " entries, above the plan's 32-bit limit";
  if (3 * nContrib > INT32_MAX)
    return "the cone units make " + std::to_string(nContrib) + " root contributions, above the plan's limit " +
           std::to_string(INT32_MAX / 3);
  return "";
}

static int64_t pushInts(std::vector<int>& pool, const std::vector<int>& v) {
  const int64_t off = (int64_t)pool.size();
  pool.insert(pool.end(), v.begin(), v.end());
  return off;
}

// 64-bit root element offsets, stored in the int pool as two ints each at an 8-byte-aligned pool
// offset (the pool is padded to an even length first; appendPools keeps the parity).
static int64_t pushOffsets(std::vector<int>& pool, const std::vector<int64_t>& v) {
  if (pool.size() & 1) pool.push_back(0);
  const int64_t off = (int64_t)pool.size();
  pool.resize(pool.size() + 2 * v.size());
  if (!v.empty()) std::memcpy(pool.data() + off, v.data(), v.size() * sizeof(int64_t));
  return off;
}

void planInstance(const cxg_problem& pr, const cxg_settings& st, Pools& pools) {
  InstanceDesc D{};
  const int n = pr.n, m = pr.m, p = pr.zero_dim, l = pr.nonneg_dim, nsoc = pr.n_soc;
  const int nr = n + p;
  // every count the device indexes with a 32-bit int (validateProblem refuses the rest first)
  const std::string lim = checkPlanCounts(pr);
  if (!lim.empty()) throw LimitError(lim);
  D.n = n; D.m = m; D.p = p; D.l = l; D.nsoc = nsoc; D.nr = nr;
  D.nnzPu = pr.Pp[n];
  D.nnzA = pr.Ap[n];
  D.pStoredNnz = pr.Pp[n];
  std::vector<int>& I = pools.ipool;

  // ---- P: full symmetric CSR over the upper entries, diagonal sources, lower root scatter ----
  std::vector<std::vector<std::pair<int, int>>> rows((size_t)n);
  std::vector<int> pdiag((size_t)n, -1), plowSrc;
  std::vector<int64_t> plowIdx;
  for (int c = 0; c < n; ++c)
    for (int k = pr.Pp[c]; k < pr.Pp[c + 1]; ++k) {
      const int r = pr.Pi[k];
      if (r > c) continue;  // below the diagonal: ignored, as the reference does
      rows[(size_t)r].push_back({c, k});
      if (r != c) {
        rows[(size_t)c].push_back({r, k});
        plowIdx.push_back(rootIdx(nr, c, r));
        plowSrc.push_back(k);
      } else if (pdiag[(size_t)c] < 0) {
        pdiag[(size_t)c] = k;
      }
    }
  std::vector<int> psRow((size_t)n + 1, 0), psCol, psSrc;
  for (int r = 0; r < n; ++r) {
    std::sort(rows[(size_t)r].begin(), rows[(size_t)r].end());
    for (auto& e : rows[(size_t)r]) { psCol.push_back(e.first); psSrc.push_back(e.second); }
    psRow[(size_t)r + 1] = (int)psCol.size();
  }
  D.nnzPs = (int)psCol.size();
  D.nPlow = (int)plowIdx.size();
  D.iPp = pushInts(I, std::vector<int>(pr.Pp, pr.Pp + n + 1));
  D.iPi = pushInts(I, std::vector<int>(pr.Pi, pr.Pi + D.nnzPu));
  D.iPsRow = pushInts(I, psRow);
  D.iPsCol = pushInts(I, psCol);
  D.iPsSrc = pushInts(I, psSrc);
  D.iPdiag = pushInts(I, pdiag);
  D.iPlowIdx = pushOffsets(I, plowIdx);
  D.iPlowSrc = pushInts(I, plowSrc);

  // ---- A: CSC (as given), CSR view, Zero-row root scatter ----
  std::vector<int> ap(pr.Ap, pr.Ap + n + 1), ai(pr.Ai, pr.Ai + D.nnzA);
  std::vector<int> arRow((size_t)m + 1, 0), arCol((size_t)D.nnzA), arSrc((size_t)D.nnzA);
  for (int k = 0; k < D.nnzA; ++k) arRow[(size_t)ai[(size_t)k] + 1]++;
  for (int r = 0; r < m; ++r) arRow[(size_t)r + 1] += arRow[(size_t)r];
  {
    std::vector<int> fill(arRow.begin(), arRow.end() - 1);
    for (int c = 0; c < n; ++c)
      for (int k = ap[(size_t)c]; k < ap[(size_t)c + 1]; ++k) {
        const int pos = fill[(size_t)ai[(size_t)k]]++;
        arCol[(size_t)pos] = c;
        arSrc[(size_t)pos] = k;
      }
  }
  std::vector<int64_t> azIdx;
  std::vector<int> azSrc;
  for (int c = 0; c < n; ++c)
    for (int k = ap[(size_t)c]; k < ap[(size_t)c + 1]; ++k)
      if (ai[(size_t)k] < p) {
        azIdx.push_back(rootIdx(nr, n + ai[(size_t)k], c));
        azSrc.push_back(k);
      }
  D.nAZ = (int)azIdx.size();
  D.iAp = pushInts(I, ap);
  D.iAi = pushInts(I, ai);
  D.iArRow = pushInts(I, arRow);
  D.iArCol = pushInts(I, arCol);
  D.iArSrc = pushInts(I, arSrc);
  D.iAZIdx = pushOffsets(I, azIdx);
  D.iAZSrc = pushInts(I, azSrc);

  // ---- cone units: NN rows then SOC blocks ----
  std::vector<int> socOff((size_t)nsoc), socDim((size_t)nsoc);
  {
    int off = p + l;
    for (int b = 0; b < nsoc; ++b) { socOff[(size_t)b] = off; socDim[(size_t)b] = pr.soc_dims[b]; off += pr.soc_dims[b]; }
  }
  D.iSocOff = pushInts(I, socOff);
  D.iSocDim = pushInts(I, socDim);
  const int nUnits = l + nsoc;
  D.nUnits = nUnits;
  std::vector<int> unitAd((size_t)nUnits + 1, 0), unitSup((size_t)nUnits + 1, 0), sup, adSrc;
  std::vector<std::pair<int64_t, int>> tgtContrib;  // (root element offset, contribution id)
  std::vector<int> contrib;                     // 3 per contribution
  for (int u = 0; u < nUnits; ++u) {
    const int r0 = (u < l) ? p + u : socOff[(size_t)(u - l)];
    const int d = (u < l) ? 1 : socDim[(size_t)(u - l)];
    std::vector<int> S;
    for (int r = r0; r < r0 + d; ++r)
      for (int k = arRow[(size_t)r]; k < arRow[(size_t)r + 1]; ++k) S.push_back(arCol[(size_t)k]);
    std::sort(S.begin(), S.end());
    S.erase(std::unique(S.begin(), S.end()), S.end());
    const int s = (int)S.size();
    const int adBase = (int)adSrc.size();
    for (int pc = 0; pc < s; ++pc)
      for (int rr = 0; rr < d; ++rr) {
        const int r = r0 + rr;
        int src = -1;
        for (int k = arRow[(size_t)r]; k < arRow[(size_t)r + 1]; ++k)
          if (arCol[(size_t)k] == S[(size_t)pc]) { src = arSrc[(size_t)k]; break; }
        adSrc.push_back(src);
      }
    for (int pi = 0; pi < s; ++pi)
      for (int pj = 0; pj <= pi; ++pj) {
        const int cid = (int)(contrib.size() / 3);
        contrib.push_back(adBase + pi * d);
        contrib.push_back(adBase + pj * d);
        contrib.push_back(d);
        tgtContrib.push_back({rootIdx(nr, S[(size_t)pi], S[(size_t)pj]), cid});
      }
    sup.insert(sup.end(), S.begin(), S.end());
    unitAd[(size_t)u + 1] = (int)adSrc.size();
    unitSup[(size_t)u + 1] = (int)sup.size();
  }
  std::stable_sort(tgtContrib.begin(), tgtContrib.end(),
                   [](const std::pair<int64_t, int>& a, const std::pair<int64_t, int>& b) { return a.first < b.first; });
  std::vector<int64_t> tgtIdx;
  std::vector<int> tgtBeg, contribSorted;
  for (size_t t = 0; t < tgtContrib.size(); ++t) {
    if (t == 0 || tgtContrib[t].first != tgtContrib[t - 1].first) {
      tgtIdx.push_back(tgtContrib[t].first);
      tgtBeg.push_back((int)(contribSorted.size() / 3));
    }
    const int cid = tgtContrib[t].second;
    contribSorted.push_back(contrib[(size_t)cid * 3 + 0]);
    contribSorted.push_back(contrib[(size_t)cid * 3 + 1]);
    contribSorted.push_back(contrib[(size_t)cid * 3 + 2]);
  }
  tgtBeg.push_back((int)(contribSorted.size() / 3));
  D.nAd = (int)adSrc.size();
  D.nTgt = (int)tgtIdx.size();
  D.nContrib = (int)(contribSorted.size() / 3);
  D.iUnitAd = pushInts(I, unitAd);
  D.iUnitSup = pushInts(I, unitSup);
  D.iSup = pushInts(I, sup);
  D.iAdSrc = pushInts(I, adSrc);
  D.iTgtIdx = pushOffsets(I, tgtIdx);
  D.iTgtBeg = pushInts(I, tgtBeg);
  D.iContrib = pushInts(I, contribSorted);

  // ---- equilibration factors ----
  std::vector<double> dv, ev;
  double c = 1.0;
  computeEquilibration(pr, st, dv, ev, c);
  D.dD = (int64_t)pools.dpool.size();
  pools.dpool.insert(pools.dpool.end(), dv.begin(), dv.end());
  D.dE = (int64_t)pools.dpool.size();
  pools.dpool.insert(pools.dpool.end(), ev.begin(), ev.end());
  D.cscale = c;

  // ---- value-array offsets (concatenated in instance order) ----
  D.vPx = pools.totPx; pools.totPx += D.nnzPu;
  D.vQ = pools.totQ; pools.totQ += n;
  D.vAx = pools.totAx; pools.totAx += D.nnzA;
  D.vB = pools.totB; pools.totB += m;
  D.vX = D.vQ;
  D.vS = D.vB;
  D.vZ = D.vB;
  D.cost = (double)nr * nr * nr / 6.0 + 30.0 * (D.nnzPs + 2.0 * D.nnzA + 9.0 * m) + 8.0 * D.nContrib;
  pools.desc.push_back(D);
}

void appendPools(Pools& dst, const Pools& src) {
  if (dst.ipool.size() & 1) dst.ipool.push_back(0);  // keeps src's 64-bit maps 8-byte aligned
  const int64_t ib = (int64_t)dst.ipool.size(), db = (int64_t)dst.dpool.size();
  dst.ipool.insert(dst.ipool.end(), src.ipool.begin(), src.ipool.end());
  dst.dpool.insert(dst.dpool.end(), src.dpool.begin(), src.dpool.end());
  for (InstanceDesc D : src.desc) {
    for (int64_t* f : {&D.iPp, &D.iPi, &D.iPsRow, &D.iPsCol, &D.iPsSrc, &D.iPdiag, &D.iPlowIdx, &D.iPlowSrc, &D.iAp,
                       &D.iAi, &D.iArRow, &D.iArCol, &D.iArSrc, &D.iAZIdx, &D.iAZSrc, &D.iSocOff, &D.iSocDim,
                       &D.iUnitAd, &D.iUnitSup, &D.iSup, &D.iAdSrc, &D.iTgtIdx, &D.iTgtBeg, &D.iContrib})
      *f += ib;
    D.dD += db;
    D.dE += db;
    D.vPx += dst.totPx;
    D.vQ += dst.totQ;
    D.vAx += dst.totAx;
    D.vB += dst.totB;
    D.vX = D.vQ;
    D.vS = D.vB;
    D.vZ = D.vB;
    dst.desc.push_back(D);
  }
  dst.totPx += src.totPx;
  dst.totQ += src.totQ;
  dst.totAx += src.totAx;
  dst.totB += src.totB;
}

}  // namespace cxg
