// Actuator-disk set-up on the host: the filtered indicator function
// (turbine_indicator.f90:43-169) and the node lists of every active
// instance's disks (turbines.f90:123-462), with the scatter windows and, for
// instances with yaw or tilt schedules, the search boxes the device
// re-evaluates each step.  Part of solver.cu's translation unit: it uses
// Derived, kPi and kPiL defined there.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <map>
#include <unordered_map>
#include <vector>

#include "lesgo_gpu.h"

namespace lesgo {

// ---------------------------------------------------------------------------
// Actuator-disk indicator (turbine_indicator.f90:43-169) and node search
// (turbines.f90:123-462), computed once on the host.
// ---------------------------------------------------------------------------
static void fft_inplace(std::complex<double>* a, int n, int stride, bool inv,
                        const std::vector<std::complex<double>>& tw) {
  // iterative radix-2 (n a power of two); tw[t] = exp(-2 pi i t / n)
  for (int i = 1, j = 0; i < n; ++i) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(a[(long long)i * stride], a[(long long)j * stride]);
  }
  for (int len = 2; len <= n; len <<= 1) {
    const int step = n / len;
    for (int i = 0; i < n; i += len)
      for (int k = 0; k < len / 2; ++k) {
        std::complex<double> w = tw[k * step];
        if (inv) w = std::conj(w);
        std::complex<double>& x = a[(long long)(i + k) * stride];
        std::complex<double>& y = a[(long long)(i + k + len / 2) * stride];
        const std::complex<double> t = y * w;
        y = x - t;
        x = x + t;
      }
  }
}

struct Indicator {
  std::vector<double> r, R2;
  double ell, thk, s6d1, M;
  double val(double rd, double x) const {
    const double rr = rd / ell, xx = x / ell;
    // linear_interp (functions.f90:712-735): clamp outside the table
    double R;
    const int N = (int)r.size();
    int i = (int)(std::upper_bound(r.begin(), r.end(), rr) - r.begin());  // r[i-1] <= rr < r[i]
    if (i == 0) R = R2[0];
    else if (i >= N) R = R2[N - 1];
    else R = R2[i - 1] + (rr - r[i - 1]) * (R2[i] - R2[i - 1]) / (r[i] - r[i - 1]);
    const double R1 = 0.5 / thk * (std::erf(s6d1 * (xx + 0.5 * thk)) - std::erf(s6d1 * (xx - 0.5 * thk)));
    return R1 * R / (ell * ell * ell);
  }
};

static Indicator make_indicator(double delta1, double delta2, double thk, double dia) {
  const int N = 2048;
  Indicator ind;
  ind.ell = 0.5 * dia;
  const double d1 = delta1 / ind.ell, d2 = delta2 / ind.ell;
  ind.thk = thk / ind.ell;
  ind.s6d1 = std::sqrt(6.0) / d1;
  const double L = 1 + 10 * d2 / std::sqrt(12.0);
  const double d = 2 * L / N;
  std::vector<double> yz(N);
  for (int i = 0; i < N; ++i) yz[i] = -L + d * ((i + 1) - 0.5);
  std::vector<std::complex<double>> g((size_t)N * N), h((size_t)N * N);
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i) {
      const double r2 = yz[i] * yz[i] + yz[j] * yz[j];
      g[(size_t)j * N + i] = 6.0 / (kPi * d2 * d2) * std::exp(-6 * r2 / (d2 * d2));
      h[(size_t)j * N + i] = (std::sqrt(r2) < 1) ? 1.0 / kPi : 0.0;
    }
  std::vector<std::complex<double>> tw(N);
  for (int t = 0; t < N; ++t) {
    const long double a = -2.0L * kPiL * t / N;
    tw[t] = std::complex<double>((double)cosl(a), (double)sinl(a));
  }
  for (auto* A : {&g, &h}) {
    for (int j = 0; j < N; ++j) fft_inplace(A->data() + (size_t)j * N, N, 1, false, tw);
    for (int i = 0; i < N; ++i) fft_inplace(A->data() + i, N, N, false, tw);
  }
  for (size_t t = 0; t < g.size(); ++t) g[t] = g[t] * h[t] * (d * d);
  for (int i = 0; i < N; ++i) fft_inplace(g.data() + i, N, N, true, tw);
  for (int j = 0; j < N; ++j) fft_inplace(g.data() + (size_t)j * N, N, 1, true, tw);
  // FFTW c2r is unnormalised: fx = N^2 (g*h d^2); R2 = fx(1, 1:N/2) / N^2
  ind.r.resize(N / 2);
  ind.R2.resize(N / 2);
  for (int jj = 0; jj < N / 2; ++jj) {
    ind.r[jj] = yz[jj] + L;
    ind.R2[jj] = g[(size_t)jj * N + 0].real() / ((double)N * N);
  }
  const double dr = ind.r[1] - ind.r[0];
  double s = 0;
  for (int jj = 0; jj < N / 2; ++jj) s += 2 * kPi * ind.r[jj] * ind.R2[jj] * dr;
  for (auto& x : ind.R2) x /= s;
  double m = 0;
  for (int jj = 0; jj < N / 2; ++jj) m += 2 * kPi * ind.r[jj] * ind.R2[jj] * ind.R2[jj] * dr;
  ind.M = m * kPi;
  return ind;
}

static long long nint_f(double x) { return x >= 0 ? (long long)std::floor(x + 0.5) : -(long long)std::floor(-x + 0.5); }

struct TurbineHost {
  int n = 0;
  std::vector<int> node_off;
  std::vector<long long> node_q;
  std::vector<double> node_ind;
  std::vector<int> win_turb;
  std::vector<long long> win_q;
  std::vector<double> win_ind;
  std::vector<long long> cols;    // (jy*ld + i) of footprint columns
  std::vector<double> nhat, ctp, corr, dia;
  std::vector<int> tinst;         // instance (slot) of each turbine
  // control schedules (turbines.f90:500-515): which*n + s -> rows / offset
  bool dyn_ctl = false, dyn_nodes = false;
  std::vector<int> s_nt, s_off;
  std::vector<double> s_t, s_v, theta, Mv;
  // the turbines of an instance with a yaw or tilt schedule take their whole
  // search box (turbines.f90:337-361) as node list, re-evaluated every step
  // on the device; the others keep the nodes selected here
  std::vector<int> dyn_list;      // box-node turbines
  std::vector<double> box_r;      // (rx, ry, rz) of each node
  std::vector<int> node_turb;     // turbine of each node
  std::vector<int> tab_off;       // indicator table of each turbine
  std::vector<double> tab_r, tab_R2, ipar;   // ipar: ell, thk, sqrt(6)/delta1, filt_max
  int tab_n = 0;
  std::vector<int> win_coff, win_cand;        // candidate box nodes of each window point
};

// Node lists of the actuator disks of every active instance, with absolute
// offsets (instance base + level*plane + jy*ld + i).  Indicator tables are
// cached by (thickness, diameter).
using IndicatorCache = std::map<std::pair<double, double>, Indicator>;
using Schedules = std::array<std::vector<double>, 3>;   // rows of theta1, theta2, Ct' (time, one value per turbine)

static TurbineHost turbines_build(const Derived& d, const std::vector<std::vector<lesgo_turbine_t>>& per_inst,
                                  const std::vector<Schedules>& sched, long long istride, IndicatorCache& cache) {
  TurbineHost th;
  const auto& P = d.p;
  const double dx = d.dx, dy = d.dy, dz = d.dz;
  const double diag = std::sqrt(dx * dx + dy * dy + dz * dz);
  const double delta1 = P.alpha1 * diag, delta2 = P.alpha2 * diag;
  const long long plane = (long long)d.ld * d.ny;
  th.node_off.push_back(0);
  std::vector<int> inst_of;
  std::vector<char> inst_box(per_inst.size(), 0);
  for (size_t inst = 0; inst < sched.size() && inst < per_inst.size(); ++inst)
    if (!sched[inst][0].empty() || !sched[inst][1].empty()) th.dyn_nodes = true, inst_box[inst] = 1;
  for (size_t inst = 0; inst < sched.size(); ++inst)
    for (int w = 0; w < 3; ++w)
      if (!sched[inst][w].empty()) th.dyn_ctl = true;
  std::vector<std::vector<int>> s_nt(3), s_off(3);
  std::map<std::pair<double, double>, int> tab_of;
  for (size_t inst = 0; inst < per_inst.size(); ++inst) {
    const long long ib = (long long)inst * istride;
    const int nloc = (int)per_inst[inst].size();
    int tl = 0;
    for (lesgo_turbine_t t : per_inst[inst]) {
      // schedule columns of this turbine
      for (int w = 0; w < 3; ++w) {
        const std::vector<double>& rows = inst < sched.size() ? sched[inst][w] : std::vector<double>();
        const int nt = rows.empty() ? 0 : (int)(rows.size() / (1 + nloc));
        s_nt[w].push_back(nt);
        s_off[w].push_back((int)th.s_t.size());
        for (int r = 0; r < nt; ++r) {
          th.s_t.push_back(rows[(size_t)r * (1 + nloc)]);
          th.s_v.push_back(rows[(size_t)r * (1 + nloc) + 1 + tl]);
        }
      }
      ++tl;
      t.thk = std::max(t.thk, dx * (double)1.01f);   // turbines.f90:180 (single-precision literal)
      auto key = std::make_pair(t.thk, t.dia);
      if (!cache.count(key)) cache[key] = make_indicator(delta1, delta2, t.thk, t.dia);
      const Indicator& ind = cache[key];
      const double search_rad = 0.5 * t.dia + 3 * std::max(P.alpha1, P.alpha2) * diag;
      const int imax = std::min((int)(search_rad / dx + 2), d.nx / 2);
      const int jmax = std::min((int)(search_rad / dy + 2), d.ny / 2);
      const double n1 = -std::cos(kPi * t.theta1 / 180.) * std::cos(kPi * t.theta2 / 180.);
      const double n2 = -std::sin(kPi * t.theta1 / 180.) * std::cos(kPi * t.theta2 / 180.);
      const double n3 = std::sin(kPi * t.theta2 / 180.);
      const long long icp = nint_f(t.xloc / dx), jcp = nint_f(t.yloc / dy);
      const double filt_max = ind.val(0.0, 0.0);
      double sumA = 0.0;
      std::vector<long long> q;
      std::vector<double> fv;
      if (th.dyn_nodes) {
        auto tk = tab_of.find(key);
        if (tk == tab_of.end()) {
          tk = tab_of.emplace(key, (int)th.tab_r.size()).first;
          th.tab_r.insert(th.tab_r.end(), ind.r.begin(), ind.r.end());
          th.tab_R2.insert(th.tab_R2.end(), ind.R2.begin(), ind.R2.end());
          th.tab_n = (int)ind.r.size();
        }
        th.tab_off.push_back(tk->second);
        th.ipar.insert(th.ipar.end(), {ind.ell, ind.thk, ind.s6d1, filt_max});
      }
      for (int k = 1; k <= d.nz; ++k) {
        if (k > d.nz_tot) continue;
        const double zt = (k - 0.5) * dz;
        for (long long j = jcp - jmax + 1; j <= jcp + jmax; ++j)
          for (long long i = icp - imax + 1; i <= icp + imax; ++i) {
            long long i2 = i, j2 = j;
            double rx, ry;
            if (i < 1) { i2 = ((i + d.nx - 1) % d.nx) + 1; rx = ((i2 - 1) * dx - P.L_x) - t.xloc; }
            else if (i > d.nx) { i2 = ((i + d.nx - 1) % d.nx) + 1; rx = (P.L_x + (i2 - 1) * dx) - t.xloc; }
            else rx = (i - 1) * dx - t.xloc;
            if (j < 1) { j2 = ((j + d.ny - 1) % d.ny) + 1; ry = ((j2 - 1) * dy - P.L_y) - t.yloc; }
            else if (j > d.ny) { j2 = ((j + d.ny - 1) % d.ny) + 1; ry = (P.L_y + (j2 - 1) * dy) - t.yloc; }
            else ry = (j - 1) * dy - t.yloc;
            const double rz = zt - t.height;
            if (inst_box[inst]) {   // every box node; the device selects them each step
              q.push_back(ib + (long long)k * plane + (j2 - 1) * d.ld + (i2 - 1));
              fv.push_back(0.0);
              th.box_r.insert(th.box_r.end(), {rx, ry, rz});
              th.node_turb.push_back(th.n);
              continue;
            }
            const double r = std::sqrt(rx * rx + ry * ry + rz * rz);
            const double r_norm = std::fabs(rx * n1 + ry * n2 + rz * n3);
            const double r_disk = std::sqrt(r * r - r_norm * r_norm);
            const double filt = ind.val(r_disk, r_norm);
            if (filt > P.filter_cutoff * filt_max) {
              q.push_back(ib + (long long)k * plane + (j2 - 1) * d.ld + (i2 - 1));
              fv.push_back(filt);
              sumA += filt * dx * dy * dz;
              if (th.dyn_nodes) {
                th.box_r.insert(th.box_r.end(), {rx, ry, rz});
                th.node_turb.push_back(th.n);
              }
            }
          }
      }
      for (size_t l = 0; l < q.size(); ++l) {
        th.node_q.push_back(q[l]);
        th.node_ind.push_back(inst_box[inst] ? 0.0 : fv[l] / sumA);
      }
      if (inst_box[inst]) th.dyn_list.push_back(th.n);
      th.theta.push_back(t.theta1);
      th.theta.push_back(t.theta2);
      th.Mv.push_back(ind.M);
      th.node_off.push_back((int)th.node_q.size());
      th.nhat.insert(th.nhat.end(), {n1, n2, n3});
      th.ctp.push_back(t.Ct_prime);
      th.corr.push_back(P.adm_correction ? (1 + 0.25 * (1 - ind.M) * t.Ct_prime) : 1.0);
      th.dia.push_back(t.dia);
      inst_of.push_back((int)inst);
      th.tinst.push_back((int)inst);
      ++th.n;
    }
  }
  // theta as [which][turbine]
  {
    std::vector<double> tt(2 * th.n);
    for (int s = 0; s < th.n; ++s) { tt[s] = th.theta[2 * s]; tt[th.n + s] = th.theta[2 * s + 1]; }
    th.theta = tt;
  }
  for (int w = 0; w < 3; ++w) {
    th.s_nt.insert(th.s_nt.end(), s_nt[w].begin(), s_nt[w].end());
    th.s_off.insert(th.s_off.end(), s_off[w].begin(), s_off[w].end());
  }
  if (th.dyn_nodes) {
    // window: every node point once (first appearance), with the nodes of
    // all turbines covering it in turbine order; the device gives a point to
    // the last turbine that selected it this step (assignment order,
    // turbines.f90:604-606) and zero to unselected points.  Static node
    // lists take part unchanged (their indicator values are positive).
    std::unordered_map<long long, int> pos;
    std::vector<std::vector<int>> cand;
    for (int s = 0; s < th.n; ++s)
      for (int l = th.node_off[s]; l < th.node_off[s + 1]; ++l) {
        auto it = pos.find(th.node_q[l]);
        if (it == pos.end()) {
          it = pos.emplace(th.node_q[l], (int)th.win_q.size()).first;
          th.win_q.push_back(th.node_q[l]);
          cand.emplace_back();
        }
        cand[it->second].push_back(l);
      }
    th.win_coff.push_back(0);
    for (auto& c : cand) {
      th.win_cand.insert(th.win_cand.end(), c.begin(), c.end());
      th.win_coff.push_back((int)th.win_cand.size());
    }
    std::unordered_map<long long, int> colset;
    for (long long q : th.win_q) {
      const long long inst = q / istride;
      const long long c = inst * istride + (q % istride) % plane;
      if (!colset.count(c)) { colset[c] = 1; th.cols.push_back(c); }
    }
    (void)inst_of;
    return th;
  }
  // scatter list: within an instance the last turbine in order owns a shared node
  std::unordered_map<long long, std::pair<int, double>> owner;
  std::vector<long long> order;
  for (int s = 0; s < th.n; ++s)
    for (int l = th.node_off[s]; l < th.node_off[s + 1]; ++l) {
      if (!owner.count(th.node_q[l])) order.push_back(th.node_q[l]);
      owner[th.node_q[l]] = {s, th.node_ind[l]};
    }
  std::unordered_map<long long, int> colset;
  for (long long q : order) {
    th.win_q.push_back(q);
    th.win_turb.push_back(owner[q].first);
    th.win_ind.push_back(owner[q].second);
    const long long inst = q / istride;
    const long long c = inst * istride + (q % istride) % plane;
    if (!colset.count(c)) { colset[c] = 1; th.cols.push_back(c); }
  }
  return th;
}

}  // namespace lesgo
