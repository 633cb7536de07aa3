// Host-side fusion planning and block-matrix construction (no device code).
//
// qsv_fusion_plan is the planner of qip_gb300/fusion.py in native code: each round
// grows up to `lookahead` candidate blocks — candidate s leaves the first s pending
// gates out and then scans in program order; a gate joins when its qubits fit (at most
// kmax) and none of them is blocked by a gate left out earlier; a left-out gate blocks
// its qubits — and keeps the candidate with the best score (first on ties): its work
// (sum of amp-update weights) plus, with lookahead2 > 0, the most work one of the
// next round's first lookahead2 candidates would take after it.  A candidate is final once it is full and all its qubits
// are blocked; prefix mode (nqubits >= 0) stops at the first round that later gates
// could still change (strict: some candidate, of either level, is not final; relaxed:
// the best is not),
// unless more than min_pending gates are pending (then the round is decided anyway).
// With beam_width or beam_branch > 1 a beam search over rounds (beam_plan) plans the
// whole list, or in prefix mode the steps taken while more than min_pending gates are
// pending.
//
// qsv_block_matrices multiplies each block's gates into its 2^k x 2^k matrix, blocks
// spread over host threads.

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "qsv_internal.cuh"

using namespace qsv;

namespace {

struct Cand {
  std::vector<int> chosen;  // positions in the pending list
  double work = 0.0;
  bool final = false;
};

void grow(const std::vector<int>& rem, int start, const uint64_t* qmask, const int* width, const double* weight,
          int kmax, int full_at, Cand& c) {
  uint64_t S = 0, blocked = 0;
  int nS = 0;
  c.chosen.clear();
  c.work = 0.0;
  c.final = false;
  const int m = (int)rem.size();
  for (int i = 0; i < m; ++i) {
    const int g = rem[(size_t)i];
    const uint64_t q = qmask[g];
    if (i < start || (q & blocked) || width[g] > kmax) {
      blocked |= q;
      if (nS >= full_at && (S & ~blocked) == 0) {
        c.final = true;
        return;
      }
      continue;
    }
    const uint64_t merged = S | q;
    const int nm = __builtin_popcountll(merged);
    if (nm <= kmax) {
      S = merged;
      nS = nm;
      c.chosen.push_back(i);
      c.work += weight[g];
    } else {
      blocked |= q;
      if (nS >= full_at && (S & ~blocked) == 0) {
        c.final = true;
        return;
      }
    }
  }
  c.final = nS >= full_at && (S & ~blocked) == 0;
}

uint64_t gate_hash(int g) {
  uint64_t z = (uint64_t)g + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Beam search over planning rounds.  A state is the list of gates not yet planned;
// each state offers its `branch` best distinct candidate blocks (most work first, ties
// to the earlier start; a gate wider than kmax at the front is a step of its own), and
// the `width` children with the least work left (ties: earlier child) form the next
// level.  Children that planned the same set of gates are merged (first kept).  Returns
// the steps of the first state that planned everything.
struct BeamState {
  std::vector<int> rem;
  double remw = 0.0;
  uint64_t key = 0;
  int node = -1;
};
struct BeamNode {
  int parent;
  std::vector<int> gates;
};

void beam_plan(const std::vector<int>& rem0, const uint64_t* qmask, const int* width, const double* weight,
               int kmax, int lookahead, int bwidth, int bbranch, std::vector<std::vector<int>>& steps) {
  std::vector<BeamNode> nodes;
  std::vector<BeamState> frontier(1);
  frontier[0].rem = rem0;
  for (int g : rem0) frontier[0].remw += weight[g];
  Cand c;
  struct Opt {
    double work;
    std::vector<int> chosen;
  };
  std::vector<Opt> opts;
  struct Child {
    int from;
    std::vector<int> chosen;
    double work;
  };
  std::vector<Child> kids;
  for (;;) {
    for (const BeamState& st : frontier)
      if (st.rem.empty()) {
        std::vector<std::vector<int>> rev;
        for (int nd = st.node; nd >= 0; nd = nodes[(size_t)nd].parent) rev.push_back(nodes[(size_t)nd].gates);
        steps.assign(rev.rbegin(), rev.rend());
        return;
      }
    kids.clear();
    for (int si = 0; si < (int)frontier.size(); ++si) {
      const std::vector<int>& rem = frontier[(size_t)si].rem;
      opts.clear();
      if (width[rem[0]] > kmax) {
        opts.push_back({weight[rem[0]], {0}});
      } else {
        const int nc = std::min<int>(lookahead, (int)rem.size());
        for (int s = 0; s < nc; ++s) {
          if (width[rem[(size_t)s]] > kmax) continue;
          grow(rem, s, qmask, width, weight, kmax, kmax, c);
          opts.push_back({c.work, c.chosen});
        }
        std::stable_sort(opts.begin(), opts.end(), [](const Opt& x, const Opt& y) { return x.work > y.work; });
      }
      int taken = 0;
      for (size_t i = 0; i < opts.size() && taken < bbranch; ++i) {
        bool dup = false;
        for (size_t j = 0; j < i && !dup; ++j) dup = opts[j].chosen == opts[i].chosen;
        if (dup) continue;
        kids.push_back({si, opts[i].chosen, opts[i].work});
        ++taken;
      }
    }
    // Merge children that planned the same gates (first kept), then keep the `width`
    // with the least work left.
    std::vector<uint64_t> keys;
    std::vector<double> remw;
    std::vector<int> kid;
    for (size_t k = 0; k < kids.size(); ++k) {
      const BeamState& st = frontier[(size_t)kids[k].from];
      uint64_t key = st.key;
      for (int i : kids[k].chosen) key += gate_hash(st.rem[(size_t)i]);
      if (std::find(keys.begin(), keys.end(), key) != keys.end()) continue;
      keys.push_back(key);
      remw.push_back(st.remw - kids[k].work);
      kid.push_back((int)k);
    }
    std::vector<int> order(kid.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return remw[(size_t)x] < remw[(size_t)y]; });
    if ((int)order.size() > bwidth) order.resize((size_t)bwidth);
    std::vector<BeamState> next;
    next.reserve(order.size());
    for (int idx : order) {
      const Child& kd = kids[(size_t)kid[(size_t)idx]];
      const BeamState& st = frontier[(size_t)kd.from];
      BeamState ns;
      ns.key = keys[(size_t)idx];
      ns.remw = remw[(size_t)idx];
      std::vector<char> picked(st.rem.size(), 0);
      BeamNode nd;
      nd.parent = st.node;
      for (int i : kd.chosen) {
        picked[(size_t)i] = 1;
        nd.gates.push_back(st.rem[(size_t)i]);
      }
      for (size_t i = 0; i < st.rem.size(); ++i)
        if (!picked[i]) ns.rem.push_back(st.rem[i]);
      ns.node = (int)nodes.size();
      nodes.push_back(std::move(nd));
      next.push_back(std::move(ns));
    }
    frontier.swap(next);
  }
}

}  // namespace

extern "C" int qsv_fusion_plan(int ngates, const uint64_t* qmask, const double* weight, int kmax, int lookahead,
                               int lookahead2, int beam_width, int beam_branch, int nqubits, int strict,
                               int min_pending, int* order_out, int* step_start_out, int* nsteps_out,
                               int* nplanned_out) {
  if (ngates < 0 || (ngates > 0 && (!qmask || !weight || !order_out || !step_start_out)) || !nsteps_out ||
      !nplanned_out || kmax < 1 || kmax > 62 || lookahead < 1 || beam_width < 1 || beam_branch < 1)
    return set_error(nullptr, QSV_ERR_INVALID, "bad fusion plan request");
  std::vector<int> width((size_t)std::max(ngates, 1));
  for (int g = 0; g < ngates; ++g) width[(size_t)g] = __builtin_popcountll(qmask[g]);
  std::vector<int> rem((size_t)ngates), next;
  for (int g = 0; g < ngates; ++g) rem[(size_t)g] = g;
  const int full_at = nqubits < 0 ? kmax : std::min(kmax, nqubits);
  int nsteps = 0, nout = 0;
  step_start_out[0] = 0;
  Cand c, best, c2;
  std::vector<int> rest2;
  // Beam search plans everything at once, or (prefix mode) the steps taken while more
  // than min_pending gates are pending; the remaining gates go through the rounds below.
  const bool use_beam = beam_width > 1 || beam_branch > 1;
  if (use_beam && !rem.empty() && (nqubits < 0 || (min_pending > 0 && (int)rem.size() > min_pending))) {
    std::vector<std::vector<int>> steps;
    beam_plan(rem, qmask, width.data(), weight, kmax, lookahead, beam_width, beam_branch, steps);
    std::vector<char> done((size_t)ngates, 0);
    int left = (int)rem.size();
    for (const auto& st : steps) {
      if (nqubits >= 0 && left <= min_pending) break;
      for (int g : st) {
        order_out[nout++] = g;
        done[(size_t)g] = 1;
      }
      step_start_out[++nsteps] = nout;
      left -= (int)st.size();
    }
    next.clear();
    for (int g : rem)
      if (!done[(size_t)g]) next.push_back(g);
    rem.swap(next);
  }
  while (!rem.empty()) {
    const int first = rem[0];
    if (width[(size_t)first] > kmax) {
      order_out[nout++] = first;
      step_start_out[++nsteps] = nout;
      rem.erase(rem.begin());
      continue;
    }
    bool have = false, undecided = false;
    double best_score = 0.0;
    // With more than min_pending gates pending the round is decided on them anyway.
    const bool forced = min_pending > 0 && (int)rem.size() > min_pending;
    const int nc = std::min<int>(lookahead, (int)rem.size());
    for (int s = 0; s < nc && !undecided; ++s) {
      if (width[(size_t)rem[(size_t)s]] > kmax) continue;
      grow(rem, s, qmask, width.data(), weight, kmax, full_at, c);
      if (nqubits >= 0 && strict && !forced && !c.final) {
        undecided = true;
        break;
      }
      // Score: the candidate's work plus the most work a next block could take after it.
      double score = c.work;
      if (lookahead2 > 0) {
        std::vector<char> in(rem.size(), 0);
        for (int i : c.chosen) in[(size_t)i] = 1;
        rest2.clear();
        for (size_t i = 0; i < rem.size(); ++i)
          if (!in[i]) rest2.push_back(rem[i]);
        double w2 = 0.0;
        const int nc2 = std::min<int>(lookahead2, (int)rest2.size());
        for (int s2 = 0; s2 < nc2; ++s2) {
          if (width[(size_t)rest2[(size_t)s2]] > kmax) continue;
          grow(rest2, s2, qmask, width.data(), weight, kmax, full_at, c2);
          if (nqubits >= 0 && strict && !forced && !c2.final) {
            undecided = true;
            break;
          }
          w2 = std::max(w2, c2.work);
        }
        score += w2;
      }
      if (undecided) break;
      if (!have || score > best_score) {
        std::swap(best, c);
        best_score = score;
        have = true;
      }
    }
    if (undecided || (nqubits >= 0 && !forced && !best.final)) break;
    std::vector<char> picked(rem.size(), 0);
    for (int i : best.chosen) {
      picked[(size_t)i] = 1;
      order_out[nout++] = rem[(size_t)i];
    }
    step_start_out[++nsteps] = nout;
    next.clear();
    for (size_t i = 0; i < rem.size(); ++i)
      if (!picked[i]) next.push_back(rem[i]);
    rem.swap(next);
  }
  *nsteps_out = nsteps;
  *nplanned_out = nout;
  return QSV_OK;
}

namespace {

// U <- G U for a gate on block bit positions bits[0..q) (bits[0] = MSB of the gate index).
void embed(int k, double* U, int q, const int* bits, const double* G) {
  const int dim = 1 << k, gd = 1 << q;
  int mask = 0;
  for (int b = 0; b < q; ++b) mask |= 1 << bits[b];
  // Diagonal gate (every off-diagonal entry exactly zero): row r of U is scaled by the
  // gate's diagonal entry at the gate index of r's bits; unit entries leave rows as
  // they are.  Same products as the general loop, without the zero terms.
  bool diagonal = true;
  for (int i = 0; i < gd && diagonal; ++i)
    for (int j = 0; j < gd; ++j)
      if (i != j && (G[2 * ((size_t)i * gd + j)] != 0.0 || G[2 * ((size_t)i * gd + j) + 1] != 0.0)) {
        diagonal = false;
        break;
      }
  if (diagonal) {
    for (int r = 0; r < dim; ++r) {
      int j = 0;
      for (int b = 0; b < q; ++b) j |= ((r >> bits[b]) & 1) << (q - 1 - b);
      const double pr = G[2 * ((size_t)j * gd + j)], pi = G[2 * ((size_t)j * gd + j) + 1];
      if (pr == 1.0 && pi == 0.0) continue;
      double* row = U + 2 * (size_t)r * dim;
      for (int c = 0; c < dim; ++c) {
        const double x = row[2 * c], y = row[2 * c + 1];
        row[2 * c] = pr * x - pi * y;
        row[2 * c + 1] = pr * y + pi * x;
      }
    }
    return;
  }
  // One qubit: rows r0 (bit clear) and r1 (bit set) combine, column by column.
  if (q == 1) {
    const int bm = 1 << bits[0];
    const double a0 = G[0], a1 = G[1], b0 = G[2], b1 = G[3], c0 = G[4], c1 = G[5], d0 = G[6], d1 = G[7];
    for (int r0 = 0; r0 < dim; ++r0) {
      if (r0 & bm) continue;
      double* x = U + 2 * (size_t)r0 * dim;
      double* y = U + 2 * (size_t)(r0 | bm) * dim;
      for (int c = 0; c < dim; ++c) {
        const double xr = x[2 * c], xi = x[2 * c + 1], yr = y[2 * c], yi = y[2 * c + 1];
        x[2 * c] = (a0 * xr - a1 * xi) + (b0 * yr - b1 * yi);
        x[2 * c + 1] = (a0 * xi + a1 * xr) + (b0 * yi + b1 * yr);
        y[2 * c] = (c0 * xr - c1 * xi) + (d0 * yr - d1 * yi);
        y[2 * c + 1] = (c0 * xi + c1 * xr) + (d0 * yi + d1 * yr);
      }
    }
    return;
  }
  std::vector<int> off((size_t)gd);
  for (int j = 0; j < gd; ++j) {
    int o = 0;
    for (int b = 0; b < q; ++b)
      if ((j >> (q - 1 - b)) & 1) o |= 1 << bits[b];
    off[(size_t)j] = o;
  }
  std::vector<double> v((size_t)2 * gd);
  for (int r0 = 0; r0 < dim; ++r0) {
    if (r0 & mask) continue;
    for (int c = 0; c < dim; ++c) {
      for (int j = 0; j < gd; ++j) {
        const double* e = U + 2 * ((size_t)(r0 | off[(size_t)j]) * dim + c);
        v[(size_t)2 * j] = e[0];
        v[(size_t)2 * j + 1] = e[1];
      }
      for (int i = 0; i < gd; ++i) {
        double re = 0.0, im = 0.0;
        const double* gi = G + 2 * (size_t)i * gd;
        for (int j = 0; j < gd; ++j) {
          const double gr = gi[2 * j], gm = gi[2 * j + 1];
          re += gr * v[(size_t)2 * j] - gm * v[(size_t)2 * j + 1];
          im += gr * v[(size_t)2 * j + 1] + gm * v[(size_t)2 * j];
        }
        double* e = U + 2 * ((size_t)(r0 | off[(size_t)i]) * dim + c);
        e[0] = re;
        e[1] = im;
      }
    }
  }
}

}  // namespace

extern "C" int qsv_block_matrices(int nblocks, const int* block_k, const int* block_qubits, const int* block_ngates,
                                  const int* gate_nq, const int* gate_qubits, const double* gate_mats,
                                  double* out) {
  if (nblocks < 0 || (nblocks > 0 && (!block_k || !block_qubits || !block_ngates || !gate_nq || !gate_qubits ||
                                      !gate_mats || !out)))
    return set_error(nullptr, QSV_ERR_INVALID, "bad block matrix request");
  // Offsets of every block's qubits, gates, gate qubits, gate matrices and output.
  std::vector<size_t> bq(nblocks + 1), bg(nblocks + 1), gq, gm, bo(nblocks + 1);
  size_t ng = 0;
  for (int b = 0; b < nblocks; ++b) {
    if (block_k[b] < 1 || block_k[b] > 10 || block_ngates[b] < 0)
      return set_error(nullptr, QSV_ERR_INVALID, "block %d: bad size", b);
    bq[b + 1] = bq[b] + (size_t)block_k[b];
    bg[b + 1] = bg[b] + (size_t)block_ngates[b];
    bo[b + 1] = bo[b] + ((size_t)2 << (2 * block_k[b]));
  }
  ng = bg[nblocks];
  gq.assign(ng + 1, 0);
  gm.assign(ng + 1, 0);
  for (size_t g = 0; g < ng; ++g) {
    if (gate_nq[g] < 1 || gate_nq[g] > 10) return set_error(nullptr, QSV_ERR_INVALID, "gate %zu: bad width", g);
    gq[g + 1] = gq[g] + (size_t)gate_nq[g];
    gm[g + 1] = gm[g] + ((size_t)2 << (2 * gate_nq[g]));
  }
  // Check every gate qubit belongs to its block before any work.
  for (int b = 0; b < nblocks; ++b)
    for (size_t g = bg[b]; g < bg[b + 1]; ++g)
      for (size_t i = gq[g]; i < gq[g + 1]; ++i) {
        bool found = false;
        for (size_t j = bq[b]; j < bq[b + 1]; ++j) found |= block_qubits[j] == gate_qubits[i];
        if (!found) return set_error(nullptr, QSV_ERR_INVALID, "block %d: gate qubit %d outside the block", b,
                                     gate_qubits[i]);
      }
  auto work = [&](int b) {
    const int k = block_k[b], dim = 1 << k;
    double* U = out + bo[(size_t)b];
    std::memset(U, 0, sizeof(double) * ((size_t)2 << (2 * k)));
    for (int i = 0; i < dim; ++i) U[2 * ((size_t)i * dim + i)] = 1.0;
    int bits[10];
    for (size_t g = bg[(size_t)b]; g < bg[(size_t)b + 1]; ++g) {
      const int q = gate_nq[g];
      for (int i = 0; i < q; ++i) {
        const int qubit = gate_qubits[gq[g] + (size_t)i];
        int pos = 0;
        while (block_qubits[bq[(size_t)b] + (size_t)pos] != qubit) ++pos;
        bits[i] = k - 1 - pos;  // block qubit 0 is the MSB of the row index
      }
      embed(k, U, q, bits, gate_mats + gm[g]);
    }
  };
  const int nthreads = std::max(1, std::min<int>(nblocks, (int)std::min(16u, std::thread::hardware_concurrency())));
  if (nthreads <= 1) {
    for (int b = 0; b < nblocks; ++b) work(b);
  } else {
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t)
      pool.emplace_back([&, t]() {
        for (int b = t; b < nblocks; b += nthreads) work(b);
      });
    for (auto& th : pool) th.join();
  }
  return QSV_OK;
}
