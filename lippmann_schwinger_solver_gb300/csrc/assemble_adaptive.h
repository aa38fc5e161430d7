// Adaptive quadtrees: the reference's default operator construction
// (GMRES/GMRES.cpp:164-199): createAdaptiveTree and createTree with
// resolveContrast (G_FMM2DTree.hpp:739-831, 891-915),
// makeLevelRestriction_Tree (:1019-1129), createCones (:1952-1974),
// assign_Tree_Interactions (:1356-1498), the NCA of getNodes_LFR /
// getNodes_HFR (:2062-2385, :3232-3571), getUserCheckPoints (:3146-3230),
// the Assemble_* block fills and getNeighbors with the precomputed
// colleague, fine, separated-fine and coarse near blocks (:1500-1950).
//
// The operator is packed into the same gather-GEMV phases as the uniform
// one (upward per level, one M2L, downward per level) and one near-field
// phase whose blocks are diag(kappa^2 q) B (+ I for the self block) of the
// leaf's neighbours; the output is P[0:N) after that phase. The phases
// follow the reference's adaptive branches: leaves on HFR levels take the
// LFR path (their own charges and M2L, potentials from every parent cone),
// HFR cones gather from leaf children directly.
//
// Included by assemble.cpp inside its anonymous namespace: it uses that
// file's quadrature, Bessel, QR, ACA and packing helpers.

class AdaptiveBuilder {
 public:
  explicit AdaptiveBuilder(const ls_config& c) : cfg(c) {}
  bool run(HostOperator& op, std::string& err);

 private:
  using Ref = std::pair<int, int>;  // (level, index in tree[level])
  struct ANode {                    // an LFR box or one cone of an HFR box
    bool out_active = false, in_active = false;
    std::vector<Ref> IL;
    std::vector<int> oc, ochk, ic, ichk, uc;  // skeleton and user check points
    std::vector<cd> Ar;             // outgoing pivot rows, rank x |sources|, row major
    long long own = -1;             // first own charge in S
    std::vector<int> fidx;          // the outgoing charges' gather indices in S
    long long pot = -1;             // first potential in P (non-leaf nodes)
  };
  struct ABox {
    int number = 0;
    double cx = 0, cy = 0, r = 0;
    bool leaf = false;
    int child[4] = {-1, -1, -1, -1};
    std::vector<Ref> nbrs;
    ANode lfr;
    std::vector<ANode> cones;
    int pt0 = -1;                                   // leaf: first of its points
    int nbr[4][20];                                 // leaf: colleague, fine, separated fine, coarse (-1: none)
  };
  static constexpr int kNbrCount[4] = {9, 12, 20, 12};
  static constexpr int kNbrLevel[4] = {0, 1, 1, -1};

  const ls_config cfg;
  int n1 = 0, rank = 0, nb = 0, nLevels = 0, level_LFR = 2, N = 0;
  double kappa = 0, L = 1, epsTree = 1e-5;
  std::vector<std::vector<ABox>> tree;
  std::vector<Ref> leaves;  // leafNodes order: the order of the points
  std::vector<double> radius, aperture, cheb1;
  std::vector<int> nCones;
  std::vector<double> L2Lc[4];  // rank x rank: a box's Chebyshev interpolant at child c's nodes
  std::vector<std::pair<int, int>> bases;
  std::vector<double> gln, glw, Qp;
  std::vector<double> gx, gy, kq;
  std::vector<int> leaf_of;     // point -> index in `leaves`
  std::map<int, std::vector<cd>> Mlev;  // leaf level -> (2S+1) x rank, [i * nS + n]
  std::map<std::tuple<int, int, int>, std::vector<cd>> nearBlk;  // (level, kind, slot) -> rank x rank, row major
  int unmatched = 0;

  double contrast(double x, double y) const { return contrast_fn(cfg, x, y); }
  ABox& box(const Ref& r) { return tree[r.first][r.second]; }
  const ABox& box(const Ref& r) const { return tree[r.first][r.second]; }
  bool lfr_box(int j, int k) const { return j >= level_LFR || tree[j][k].leaf; }

  // ---- tree ------------------------------------------------------------------
  // getS / get_Transfer_Matrix (:675-681, :725-737): the interpolation of a
  // box's nodal values to its children's nodes.
  void cheb_setup() {
    for (int k = 0; k < n1; ++k) cheb1.push_back(-std::cos((k + 0.5) / n1 * kPi));
    auto getS = [&](double x, double y) {
      double s = 0.5;
      for (int k = 1; k < n1; ++k) s += cheb_t(x, k) * cheb_t(y, k);
      return 2.0 / n1 * s;
    };
    const double sx[4] = {-0.5, 0.5, 0.5, -0.5}, sy[4] = {-0.5, -0.5, 0.5, 0.5};
    for (int c = 0; c < 4; ++c) {
      L2Lc[c].assign((size_t)rank * rank, 0.0);
      for (int j = 0; j < rank; ++j)
        for (int k = 0; k < rank; ++k) {
          const double chx = 0.5 * cheb1[j % n1] + sx[c], chy = 0.5 * cheb1[j / n1] + sy[c];
          L2Lc[c][(size_t)j * rank + k] = getS(cheb1[k % n1], chx) * getS(cheb1[k / n1], chy);
        }
    }
  }
  // resolveContrast (:739-754): max error of the box's Chebyshev interpolant
  // of q at its children's nodes.
  double resolve_contrast(const ABox& B) const {
    std::vector<double> qn(rank);
    for (int i = 0; i < rank; ++i) qn[i] = contrast(B.r * cheb1[i % n1] + B.cx, B.r * cheb1[i / n1] + B.cy);
    const double sx[4] = {-0.5, 0.5, 0.5, -0.5}, sy[4] = {-0.5, -0.5, 0.5, 0.5};
    double e = 0.0;
    std::vector<double> approx(4 * rank), truth(4 * rank);
    for (int c = 0; c < 4; ++c)
      for (int j = 0; j < rank; ++j) {
        double s = 0.0;
        for (int k = 0; k < rank; ++k) s += L2Lc[c][(size_t)j * rank + k] * qn[k];
        approx[c * rank + j] = s;
        const double chx = 0.5 * cheb1[j % n1] + sx[c], chy = 0.5 * cheb1[j / n1] + sy[c];
        truth[c * rank + j] = contrast(B.r * chx + B.cx, B.r * chy + B.cy);
      }
    for (int i = 0; i < 4 * rank; ++i) e = std::max(e, std::fabs(truth[i] - approx[i]));
    return e;
  }
  void add_children(int j, int k) {
    if ((int)tree.size() == j + 1) tree.emplace_back();
    const ABox P = tree[j][k];
    const double h = 0.5 * P.r;
    for (int c = 0; c < 4; ++c) {
      ABox B;
      B.number = P.number * 4 + c;
      B.r = 0.5 * P.r;
      B.cx = (c == 0 || c == 3) ? P.cx - h : P.cx + h;
      B.cy = (c == 0 || c == 1) ? P.cy - h : P.cy + h;
      tree[j][k].child[c] = (int)tree[j + 1].size();
      tree[j + 1].push_back(B);
    }
  }
  // createTree (:773-831): split while q is not resolved to epsilonTree or
  // the box spans more than one wavelength.
  void create_tree(int j, int k) {
    const bool c1 = resolve_contrast(tree[j][k]) < epsTree;
    const bool c3 = kappa * tree[j][k].r / 2 / kPi <= 1.0;
    if (c1 && c3) {
      tree[j][k].leaf = true;
      leaves.push_back({j, k});
      return;
    }
    add_children(j, k);
    for (int c = 0; c < 4; ++c) create_tree(j + 1, tree[j][k].child[c]);
  }
  bool adjacent(int bj, int bk, int nj, int nk) const {
    const double epsR = 1e-8;
    const ABox& A = tree[bj][bk];
    const ABox& O = tree[nj][nk];
    return !(std::fabs(A.cx - O.cx) >= 3.0 * radius[bj] + radius[nj] - epsR ||
             std::fabs(A.cy - O.cy) >= 3.0 * radius[bj] + radius[nj] - epsR);
  }
  // getFutureGeneration_LFR (:943-964): the leaf descendants of (pj, pk)
  // adjacent to (bj, bk).
  void future_generation(int bj, int bk, int pj, int pk, std::vector<Ref>& out) const {
    if (tree[pj][pk].leaf) {
      if (adjacent(bj, bk, pj, pk)) out.push_back({pj, pk});
      return;
    }
    for (int c = 0; c < 4; ++c) future_generation(bj, bk, pj + 1, tree[pj][pk].child[c], out);
  }
  // makeLevelRestriction_Tree (:1019-1129): refine a leaf whose neighbour
  // list holds a leaf two or more levels finer, nLevels passes.
  void level_restriction() {
    for (int pass = 0; pass < nLevels; ++pass) {
      std::vector<std::vector<std::vector<Ref>>> nbl(nLevels + 1);
      for (int j = 0; j <= nLevels; ++j) nbl[j].assign(tree[j].size(), {});
      for (int c = 0; c < 4; ++c)
        for (int n = 0; n < 4; ++n) nbl[1][c].push_back({1, n});
      for (int j = 1; j <= nLevels - 1; ++j)
        for (int k = 0; k < (int)tree[j].size(); ++k) {
          if (tree[j][k].leaf) continue;
          for (int c = 0; c < 4; ++c) {
            const int A = tree[j][k].child[c];
            for (const Ref& p : nbl[j][k]) {
              std::vector<Ref> fg;
              future_generation(j + 1, A, p.first, p.second, fg);
              nbl[j + 1][A].insert(nbl[j + 1][A].end(), fg.begin(), fg.end());
            }
          }
        }
      std::vector<Ref> old = leaves;
      auto index_of = [&](Ref p) {
        for (size_t l = 0; l < leaves.size(); ++l)
          if (leaves[l] == p) return (int)l;
        return -1;
      };
      auto refine = [&](int l, Ref leaf) {
        old[l].first = -1;
        tree[leaf.first][leaf.second].leaf = false;
        add_children(leaf.first, leaf.second);
        for (int c = 0; c < 4; ++c) {
          const int ch = tree[leaf.first][leaf.second].child[c];
          tree[leaf.first + 1][ch].leaf = true;
          leaves.push_back({leaf.first + 1, ch});
        }
      };
      for (size_t l = 0; l < old.size(); ++l) {
        const Ref leaf = leaves[l];
        for (const Ref& p : nbl[leaf.first][leaf.second]) {
          if (leaf.first - p.first >= 2) {
            const int id = index_of(p);
            if (id >= 0 && old[id].first != -1) refine(id, p);
          } else if (p.first - leaf.first >= 2) {
            if (old[l].first != -1) refine((int)l, leaf);
          }
        }
      }
      int cnt = 0;
      for (size_t l = 0; l < old.size(); ++l)
        if (old[l].first == -1) {
          leaves.erase(leaves.begin() + l - cnt);
          ++cnt;
        }
    }
  }
  // assign_Child_Interaction (:1356-1461).
  void child_interactions(int c, int j, int k) {
    const double epsR = 1e-8;
    const int A = tree[j][k].child[c];
    ABox& BA = tree[j + 1][A];
    const std::vector<Ref> pn = tree[j][k].nbrs;
    for (const Ref& p : pn) {
      const int pj = p.first, pk = p.second;
      if (j + 1 >= level_LFR || BA.leaf) {
        if (tree[pj][pk].leaf) {
          if (!adjacent(j + 1, A, pj, pk)) BA.lfr.IL.push_back(p);
          else BA.nbrs.push_back(p);
        } else {
          for (int nc = 0; nc < 4; ++nc) {
            const int Bk = tree[pj][pk].child[nc];
            if (!adjacent(j + 1, A, pj + 1, Bk)) {
              BA.lfr.IL.push_back({pj + 1, Bk});
            } else if (!BA.leaf) {
              BA.nbrs.push_back({pj + 1, Bk});
            } else {
              std::vector<Ref> fg;
              future_generation(j + 1, A, pj + 1, Bk, fg);
              BA.nbrs.insert(BA.nbrs.end(), fg.begin(), fg.end());
            }
          }
        }
      } else {
        const double r = radius[j + 1];
        auto cone_of = [&](const ABox& O) {
          double arg = std::atan2(BA.cy - O.cy, BA.cx - O.cx);
          arg = std::fmod(arg + 2 * kPi + kPi, 2 * kPi);
          return int(arg / aperture[j + 1]);
        };
        if (tree[pj][pk].leaf) {
          const ABox& O = tree[pj][pk];
          if (std::fabs(BA.cx - O.cx) >= kappa * r * r + r + radius[pj] - epsR ||
              std::fabs(BA.cy - O.cy) >= kappa * r * r + r + radius[pj] - epsR)
            BA.cones[cone_of(O)].IL.push_back(p);
          else
            BA.nbrs.push_back(p);
        } else {
          for (int nc = 0; nc < 4; ++nc) {
            const int Bk = tree[pj][pk].child[nc];
            const ABox& O = tree[pj + 1][Bk];
            // the y test omits the target's radius, as the reference's (:1441-1442)
            if (std::fabs(BA.cx - O.cx) >= kappa * r * r + r + radius[pj + 1] - epsR ||
                std::fabs(BA.cy - O.cy) >= kappa * r * r + radius[pj + 1] - epsR)
              BA.cones[cone_of(O)].IL.push_back({pj + 1, Bk});
            else
              BA.nbrs.push_back({pj + 1, Bk});
          }
        }
      }
    }
  }

  // ---- precomputations -------------------------------------------------------
  void precompute_Q() {
    std::vector<cd> Q((size_t)rank * nb);
    for (int l = 0; l < nb; ++l)
      for (int i = 0; i < rank; ++i)
        Q[(size_t)l * rank + i] =
            cd(cheb_t(cheb1[i % n1], bases[l].first) * cheb_t(cheb1[i / n1], bases[l].second), 0.0);
    PivQR qr;
    qr.factor(rank, nb, Q);
    Qp.assign((size_t)nb * rank, 0.0);
    std::vector<cd> e(rank), s(nb);
    for (int i = 0; i < rank; ++i) {
      std::fill(e.begin(), e.end(), cd(0.0, 0.0));
      e[i] = 1.0;
      qr.solve(e.data(), s.data());
      for (int l = 0; l < nb; ++l) Qp[(size_t)l * rank + i] = s[l].real();
    }
  }
  // FarFieldInteraction::evaluateC/M (FarFieldInteraction.hpp:115-160) at a
  // leaf level, rounded like the text cache.
  void precompute_M(int j) {
    const int nS = 2 * kSeries + 1;
    const double rj = radius[j];
    std::vector<cd> C((size_t)nS * nb);
#pragma omp parallel for schedule(dynamic, 1)
    for (int t = 0; t < nS * nb; ++t) {
      const int n = t / nb - kSeries, l = t % nb;
      const int a = bases[l].first, b = bases[l].second;
      auto f = [&](double x, double y) -> cd {
        const double R2 = x * x + y * y;
        const double nx = std::sqrt(R2);
        const double arg = kappa * rj * nx;
        const double th = std::atan2(y, x);
        return bes_j(n, arg) * std::exp(-kI * double(n) * th) * cheb_t(x, a) * cheb_t(y, b);
      };
      C[(size_t)(n + kSeries) * nb + l] = rj * rj * quad2d(f, gln, glw);
    }
    finish_M(j, C);
  }
  // M = C Q^+ of leaf level j, rounded like the text cache.
  void finish_M(int j, const std::vector<cd>& C) {
    const int nS = 2 * kSeries + 1;
    std::vector<cd> M((size_t)nS * rank);
    for (int n = 0; n < nS; ++n)
      for (int i = 0; i < rank; ++i) {
        cd s(0.0, 0.0);
        for (int l = 0; l < nb; ++l) s += C[(size_t)n * nb + l] * Qp[(size_t)l * rank + i];
        if (cfg.reference_rounding) s = cd(round6(s.real()), round6(s.imag()));
        M[(size_t)i * nS + n] = s;
      }
    Mlev[j] = std::move(M);
  }

  // ---- far-field entries (getMatrixEntry :603-658) -----------------------------
  // Per-task cache of sum_n M[node][n] h_n of a target about a source leaf,
  // for all rank source nodes of the leaf.
  struct HCache {
    const AdaptiveBuilder* b;
    std::unordered_map<long long, std::vector<cd>> m;
    const cd* get(int i, int leaf) {
      const long long key = (long long)i * 1048576LL + leaf;
      auto it = m.find(key);
      if (it != m.end()) return it->second.data();
      const ABox& B = b->box(b->leaves[leaf]);
      const double rx = b->gx[i] - B.cx, ry = b->gy[i] - B.cy;
      const double th = std::atan2(ry, rx);
      const double R = b->kappa * std::sqrt(ry * ry + rx * rx);
      double J[kSeries + 1], Y[kSeries + 1];
      bessel_jy_orders(kSeries, R, J, Y);
      constexpr int nS = 2 * kSeries + 1;
      cd h[nS];
      for (int n = -kSeries; n <= kSeries; ++n) {
        const int a = n < 0 ? -n : n;
        const double sg = (n < 0 && (a % 2 == 1)) ? -1.0 : 1.0;
        const double jn = sg == 1.0 ? J[a] : -J[a];
        const double yn = sg == 1.0 ? Y[a] : -Y[a];
        h[n + kSeries] = (jn + kI * yn) * std::exp(kI * double(n) * th);
      }
      const std::vector<cd>& M = b->Mlev.at(b->leaves[leaf].first);
      std::vector<cd> out(b->rank);
      for (int idx = 0; idx < b->rank; ++idx) {
        cd s = 0.0 + 0.0 * kI;
        for (int n = 0; n < nS; ++n) s += M[(size_t)idx * nS + n] * h[n];
        out[idx] = s;
      }
      return m.emplace(key, std::move(out)).first->second.data();
    }
  };
  cd entry(int i, int j, HCache& hc) const {
    cd s = hc.get(i, leaf_of[j])[j % rank];
    s *= kI / 4.0;
    if (cfg.findPhi) {
      s *= kq[i];
      if (i == j) s += 1.0;
    }
    return s;
  }
  // Row-major K(rows, cols).
  std::vector<cd> block(const std::vector<int>& rows, const std::vector<int>& cols, HCache& hc) const {
    std::vector<cd> A(rows.size() * cols.size());
    for (size_t a = 0; a < rows.size(); ++a)
      for (size_t c = 0; c < cols.size(); ++c) A[a * cols.size() + c] = entry(rows[a], cols[c], hc);
    return A;
  }
  int aca(const std::vector<int>& rows, const std::vector<int>& cols, double eps, std::vector<int>& rb,
          std::vector<int>& cb, std::vector<cd>* Ar, HCache& hc) const {
    const int n1r = (int)rows.size(), n2 = (int)cols.size();
    auto get_row = [&](int r) { std::vector<cd> o(n2); for (int k = 0; k < n2; ++k) o[k] = entry(rows[r], cols[k], hc); return o; };
    auto get_col = [&](int c) { std::vector<cd> o(n1r); for (int k = 0; k < n1r; ++k) o[k] = entry(rows[k], cols[c], hc); return o; };
    return aca_core(n1r, n2, eps, rb, cb, Ar, get_row, get_col);
  }

  // ---- NCA (getNodes_LFR / getNodes_HFR) -------------------------------------
  // Points a node offers to a parent / an interaction partner: a leaf's own
  // points; else its children's (LFR children whole, HFR children through
  // the cone of the relation: all of their cones, or cone / 2).
  std::vector<int> own_points(int j, int k, int cone, bool outgoing) const {
    const ABox& B = tree[j][k];
    if (B.leaf) {
      std::vector<int> v(rank);
      for (int i = 0; i < rank; ++i) v[i] = B.pt0 + i;
      return v;
    }
    std::vector<int> out;
    for (int c = 0; c < 4; ++c) {
      const ABox& ch = tree[j + 1][B.child[c]];
      auto take = [&](const ANode& n) {
        const std::vector<int>& v = outgoing ? n.oc : n.ichk;
        out.insert(out.end(), v.begin(), v.end());
      };
      if (cone < 0) {  // an LFR box: children whole
        if (lfr_box(j + 1, B.child[c])) take(ch.lfr);
        else for (const ANode& cn : ch.cones) take(cn);
      } else {
        if (j == level_LFR - 1 || ch.leaf) take(ch.lfr);
        else take(ch.cones[cone / 2]);
      }
    }
    return out;
  }
  // Cone of box (ja, ka) that points at box (j, k) (:2524-2526, :3335-3337).
  int cone_towards(int j, int k, int ja, int ka) const {
    const double arg = std::atan2(tree[j][k].cy - tree[ja][ka].cy, tree[j][k].cx - tree[ja][ka].cx);
    return int(std::fmod(arg + 2 * kPi, 2 * kPi) / aperture[ja]);
  }
  const ANode& partner(const Ref& p, int j, int k) const {
    const ABox& O = box(p);
    if (p.first < level_LFR && !O.leaf) return O.cones[cone_towards(j, k, p.first, p.second)];
    return O.lfr;
  }
  void nca_node(int j, int k, int cone, bool outgoing, double tol) {
    ABox& B = tree[j][k];
    ANode& nd = cone < 0 ? B.lfr : B.cones[cone];
    HCache hc{this, {}};
    const std::vector<int> own = own_points(j, k, cone, outgoing);
    std::vector<int> far;
    for (const Ref& p : nd.IL) {
      std::vector<int> v;
      if (cone < 0) {
        v = box(p).leaf ? own_points(p.first, p.second, -1, !outgoing)
                        : own_points(p.first, p.second, -1, !outgoing);
      } else {
        const ABox& O = box(p);
        v = O.leaf ? own_points(p.first, p.second, -1, !outgoing)
                   : own_points(p.first, p.second, cone_towards(j, k, p.first, p.second), !outgoing);
      }
      far.insert(far.end(), v.begin(), v.end());
    }
    std::vector<int> rb, cb;
    if (outgoing) {
      if (!far.empty() && !own.empty()) {
        nd.out_active = true;
        const int rk = aca(far, own, tol, rb, cb, &nd.Ar, hc);
        if (rk > 0) {
          for (int r : rb) nd.ochk.push_back(far[r]);
          for (int c : cb) nd.oc.push_back(own[c]);
        }
      } else {
        nd.out_active = false;
        nd.oc = own;
      }
    } else {
      if (!far.empty() && !own.empty()) {
        nd.in_active = true;
        const int rk = aca(own, far, tol, rb, cb, nullptr, hc);
        if (rk > 0) {
          for (int r : rb) nd.ichk.push_back(own[r]);
          for (int c : cb) nd.ic.push_back(far[c]);
        }
      } else {
        nd.in_active = false;
        nd.ichk = own;
      }
    }
  }
  void nca() {
    const double tol = std::pow(10, -1.0 * cfg.TOL_POW);
    for (int j = nLevels; j >= 2; --j) {
      std::vector<std::pair<int, int>> work;
      for (int k = 0; k < (int)tree[j].size(); ++k) {
        if (lfr_box(j, k)) work.push_back({k, -1});
        else for (int c = 0; c < nCones[j]; ++c) work.push_back({k, c});
      }
      for (int dir = 0; dir < 2; ++dir) {
#pragma omp parallel for schedule(dynamic, 1)
        for (int t = 0; t < (int)work.size(); ++t) nca_node(j, work[t].first, work[t].second, dir == 0, tol);
      }
    }
  }
  // getUserCheckPoints (:3146-3230).
  void user_checks() {
    for (int j = nLevels; j >= 2; --j)
      for (int k = 0; k < (int)tree[j].size(); ++k) {
        ABox& B = tree[j][k];
        if (B.leaf) {
          for (int i = 0; i < rank; ++i) B.lfr.uc.push_back(B.pt0 + i);
          continue;
        }
        if (j >= level_LFR) {
          if (B.lfr.in_active) B.lfr.uc = B.lfr.ichk;
          else for (int c = 0; c < 4; ++c) { const auto& v = tree[j + 1][B.child[c]].lfr.uc; B.lfr.uc.insert(B.lfr.uc.end(), v.begin(), v.end()); }
          continue;
        }
        for (int cone = 0; cone < nCones[j]; ++cone) {
          ANode& C = B.cones[cone];
          if (C.in_active) { C.uc = C.ichk; continue; }
          for (int c = 0; c < 4; ++c) {
            const ABox& ch = tree[j + 1][B.child[c]];
            const auto& v = (ch.leaf || j + 1 == level_LFR) ? ch.lfr.uc : ch.cones[cone / 2].uc;
            C.uc.insert(C.uc.end(), v.begin(), v.end());
          }
        }
      }
  }

  // ---- near field --------------------------------------------------------------
  // Neighbour offsets in units of the leaf's radius (N_centers, FN_centers,
  // SFN_centers, CN_centers): the self box is the last colleague.
  static std::vector<std::pair<double, double>> offsets(int kind) {
    std::vector<std::pair<double, double>> v;
    if (kind == 0) {
      for (int a = -1; a <= 1; ++a)
        for (int b = -1; b <= 1; ++b)
          if (a || b) v.push_back({2.0 * a, 2.0 * b});
      v.push_back({0.0, 0.0});
      return v;
    }
    const double e1[4] = {-1.5, -0.5, 0.5, 1.5}, e2[6] = {-2.5, -1.5, -0.5, 0.5, 1.5, 2.5},
                 e3[4] = {-3.0, -1.0, 1.0, 3.0};
    const double* e = kind == 1 ? e1 : kind == 2 ? e2 : e3;
    const int ne = kind == 2 ? 6 : 4;
    const double edge = kind == 1 ? 1.5 : kind == 2 ? 2.5 : 3.0;
    for (int a = 0; a < ne; ++a)
      for (int b = 0; b < ne; ++b)
        if (std::fabs(e[a]) == edge || std::fabs(e[b]) == edge) v.push_back({e[a], e[b]});
    return v;
  }
  // getNeighbors (:1500-1748); separated fine neighbours are the finer ones
  // farther than 2.5 radii (find_distance :1350).
  void classify_neighbors() {
    std::vector<std::pair<double, double>> tab[4] = {offsets(0), offsets(1), offsets(2), offsets(3)};
    for (const Ref& lf : leaves) {
      ABox& B = box(lf);
      for (auto& row : B.nbr) std::fill(row, row + 20, -1);
      const double r = radius[lf.first];
      for (const Ref& p : B.nbrs) {
        const ABox& O = box(p);
        const double dx = (O.cx - B.cx) / r, dy = (O.cy - B.cy) / r;
        int kind;
        if (p.first == lf.first) kind = 0;
        else if (p.first == lf.first + 1) kind = std::sqrt(dx * dx + dy * dy) > 2.5 ? 2 : 1;
        else if (p.first == lf.first - 1) kind = 3;
        else { ++unmatched; continue; }
        int found = -1;
        for (size_t t = 0; t < tab[kind].size(); ++t)
          if (std::fabs(tab[kind][t].first - dx) < 1e-8 && std::fabs(tab[kind][t].second - dy) < 1e-8) found = (int)t;
        if (found < 0) { ++unmatched; continue; }
        B.nbr[kind][found] = p.second;
      }
    }
  }
  // getOperator (:1773-1806) with NearFieldInteraction1::evaluateV: target
  // box of radius rA at the origin, source box of radius rB at (cx, cy).
  std::vector<cd> near_block(double rA, double rB, double cx, double cy) const {
    std::vector<cd> V((size_t)rank * nb);
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < rank; ++i) {
      const double Xx = (rA * cheb1[i % n1] - cx) / rB, Xy = (rA * cheb1[i / n1] - cy) / rB;
      for (int l = 0; l < nb; ++l) {
        const int a = bases[l].first, b = bases[l].second;
        auto f = [&](double px, double py) -> cd {
          const double R2 = (Xx - px) * (Xx - px) + (Xy - py) * (Xy - py);
          const double R = std::sqrt(R2);
          const double arg = kappa * rB * R;
          return (bes_j(0, arg) + kI * bes_y(0, arg)) * cheb_t(px, a) * cheb_t(py, b);
        };
        V[(size_t)i * nb + l] = quad2d(f, gln, glw);
      }
    }
    return finish_near(rB, V);
  }
  // Bk = V (i rB^2 / 4) Q^+, rounded like the text cache.
  std::vector<cd> finish_near(double rB, const std::vector<cd>& V) const {
    std::vector<cd> Bk((size_t)rank * rank);
    for (int i = 0; i < rank; ++i)
      for (int k = 0; k < rank; ++k) {
        cd s(0.0, 0.0);
        for (int l = 0; l < nb; ++l) s += V[(size_t)i * nb + l] * kI * rB * rB / 4.0 * Qp[(size_t)l * rank + k];
        Bk[(size_t)i * rank + k] = cfg.reference_rounding ? cd(round6(s.real()), round6(s.imag())) : s;
      }
    return Bk;
  }
  // Every leaf level's far moments and every near block in one GPU batch
  // (csrc/quadrature.cu); false when there is no GPU for it (the host
  // routines above then run).
  bool precompute_on_gpu(const std::set<int>& leaf_levels) {
    const int dev = quadrature_device(cfg);
    if (dev < 0) return false;
    const int nS = 2 * kSeries + 1;
    std::vector<QuadTask> tasks;
    std::vector<int> levels;
    for (int j : leaf_levels)
      if (!Mlev.count(j)) levels.push_back(j);
    for (int j : levels)
      for (int t = 0; t < nS * nb; ++t)
        tasks.push_back({0.0, 0.0, kappa * radius[j], bases[t % nb].first, bases[t % nb].second, t / nb - kSeries, 1});
    std::vector<std::pair<double, double>> tab[4] = {offsets(0), offsets(1), offsets(2), offsets(3)};
    struct NearKey { std::tuple<int, int, int> key; double rB; };
    std::vector<NearKey> keys;
    std::set<std::tuple<int, int, int>> seen;
    for (const Ref& lf : leaves) {
      const ABox& B = box(lf);
      for (int kind = 0; kind < 4; ++kind)
        for (int t = 0; t < kNbrCount[kind]; ++t) {
          if (B.nbr[kind][t] < 0) continue;
          const auto key = std::make_tuple(lf.first, kind, t);
          if (nearBlk.count(key) || !seen.insert(key).second) continue;
          const double rA = radius[lf.first], rB = radius[lf.first + kNbrLevel[kind]];
          const double cx = tab[kind][t].first * rA, cy = tab[kind][t].second * rA;
          keys.push_back({key, rB});
          for (int i = 0; i < rank; ++i) {
            const double Xx = (rA * cheb1[i % n1] - cx) / rB, Xy = (rA * cheb1[i / n1] - cy) / rB;
            for (int l = 0; l < nb; ++l) tasks.push_back({Xx, Xy, kappa * rB, bases[l].first, bases[l].second, 0, 0});
          }
        }
    }
    std::vector<cd> qv;
    if (tasks.empty()) return true;
    if (!gpu_quadrature(dev, tasks, gln, glw, qv)) return false;
    size_t o = 0;
    for (int j : levels) {
      const double rj = radius[j];
      std::vector<cd> C((size_t)nS * nb);
      for (int t = 0; t < nS * nb; ++t) C[t] = rj * rj * qv[o + t];
      o += (size_t)nS * nb;
      finish_M(j, C);
    }
    for (const NearKey& k : keys) {
      std::vector<cd> V(qv.begin() + o, qv.begin() + o + (size_t)rank * nb);
      o += (size_t)rank * nb;
      nearBlk[k.key] = finish_near(k.rB, V);
    }
    return true;
  }
  // Precomputation-cache keys of a leaf level's far moments and of a near
  // block (level, kind, slot), for host (gpu 0) or GPU (1) integration.
  std::string m_key(int j, int gpu) const {
    return pc_key("adaptive-M", {kappa, radius[j]}, {n1, cfg.degreeOfBases, cfg.reference_rounding, gpu, kSeries});
  }
  std::string near_key(const std::tuple<int, int, int>& key, const std::vector<std::pair<double, double>>* tab,
                       int gpu) const {
    const int j = std::get<0>(key), kind = std::get<1>(key), t = std::get<2>(key);
    const double rA = radius[j], rB = radius[j + kNbrLevel[kind]];
    return pc_key("adaptive-near", {kappa, rA, rB, tab[kind][t].first * rA, tab[kind][t].second * rA},
                  {n1, cfg.degreeOfBases, cfg.reference_rounding, gpu});
  }
  // The leaf levels' moments and the near blocks the leaves use: read from
  // the precomputation cache what it holds, integrate the rest (on the GPU
  // when so configured, else on the host), and store what was integrated.
  void precomputations(const std::set<int>& leaf_levels) {
    std::vector<std::pair<double, double>> tab[4] = {offsets(0), offsets(1), offsets(2), offsets(3)};
    std::set<std::tuple<int, int, int>> used;
    for (const Ref& lf : leaves) {
      const ABox& B = box(lf);
      for (int kind = 0; kind < 4; ++kind)
        for (int t = 0; t < kNbrCount[kind]; ++t)
          if (B.nbr[kind][t] >= 0) used.insert(std::make_tuple(lf.first, kind, t));
    }
    const int want_gpu = quadrature_device(cfg) >= 0 ? 1 : 0;
    std::set<int> cached_m;
    std::set<std::tuple<int, int, int>> cached_near;
    if (g_pcache.enabled()) {
      std::vector<cd> rec;
      for (int j : leaf_levels)
        if (g_pcache.get(m_key(j, want_gpu), rec) && rec.size() == (size_t)(2 * kSeries + 1) * rank) {
          Mlev[j] = rec;
          cached_m.insert(j);
        }
      for (const auto& key : used)
        if (g_pcache.get(near_key(key, tab, want_gpu), rec) && rec.size() == (size_t)rank * rank) {
          nearBlk[key] = rec;
          cached_near.insert(key);
        }
    }
    const bool gpu = precompute_on_gpu(leaf_levels);
    if (!gpu) {
      for (int j : leaf_levels)
        if (!Mlev.count(j)) precompute_M(j);
      precompute_near();
    }
    if (g_pcache.enabled()) {
      for (int j : leaf_levels)
        if (!cached_m.count(j)) g_pcache.put(m_key(j, gpu ? 1 : 0), Mlev.at(j));
      for (const auto& key : used)
        if (!cached_near.count(key)) g_pcache.put(near_key(key, tab, gpu ? 1 : 0), nearBlk.at(key));
    }
  }
  void precompute_near() {
    std::vector<std::pair<double, double>> tab[4] = {offsets(0), offsets(1), offsets(2), offsets(3)};
    for (const Ref& lf : leaves) {
      const ABox& B = box(lf);
      for (int kind = 0; kind < 4; ++kind)
        for (int t = 0; t < kNbrCount[kind]; ++t) {
          if (B.nbr[kind][t] < 0) continue;
          const auto key = std::make_tuple(lf.first, kind, t);
          if (nearBlk.count(key)) continue;
          const double rA = radius[lf.first], rB = radius[lf.first + kNbrLevel[kind]];
          nearBlk[key] = near_block(rA, rB, tab[kind][t].first * rA, tab[kind][t].second * rA);
        }
    }
  }

  void pack(HostOperator& op);
};

constexpr int AdaptiveBuilder::kNbrCount[4];
constexpr int AdaptiveBuilder::kNbrLevel[4];

// W x = Atilde^{-1} applied on the right, row by row through a QR of
// Atilde^T (see the uniform downward pass), for an r x r Atilde.
static void fold_right_inverse(const std::vector<cd>& Lb, int rows, int r, const PivQR& AT, std::vector<cd>& W) {
  W.assign((size_t)rows * r, cd(0.0, 0.0));
  for (int a = 0; a < rows; ++a) AT.solve(&Lb[(size_t)a * r], &W[(size_t)a * r]);
}

void AdaptiveBuilder::pack(HostOperator& op) {
  // ---- charges S: x, then own skeleton charges (children before parents).
  long long S = N;
  for (int j = nLevels; j >= 2; --j)
    for (int k = 0; k < (int)tree[j].size(); ++k) {
      ABox& B = tree[j][k];
      if (lfr_box(j, k)) {
        if (B.lfr.out_active && !B.lfr.oc.empty()) { B.lfr.own = S; S += (long long)B.lfr.oc.size(); }
      } else {
        for (ANode& C : B.cones)
          if (C.out_active && !C.oc.empty()) { C.own = S; S += (long long)C.oc.size(); }
      }
    }
  // Gather lists of the outgoing charges, bottom up.
  for (int j = nLevels; j >= 2; --j)
    for (int k = 0; k < (int)tree[j].size(); ++k) {
      ABox& B = tree[j][k];
      if (lfr_box(j, k)) {
        ANode& nd = B.lfr;
        nd.fidx.clear();
        if (nd.out_active) {
          for (size_t s = 0; s < nd.oc.size(); ++s) nd.fidx.push_back((int)(nd.own + (long long)s));
        } else if (B.leaf) {
          for (int i = 0; i < rank; ++i) nd.fidx.push_back(B.pt0 + i);
        } else {
          for (int c = 0; c < 4; ++c) { const auto& v = tree[j + 1][B.child[c]].lfr.fidx; nd.fidx.insert(nd.fidx.end(), v.begin(), v.end()); }
        }
      } else {
        for (int cone = 0; cone < nCones[j]; ++cone) {
          ANode& C = B.cones[cone];
          C.fidx.clear();
          if (C.out_active) {
            for (size_t s = 0; s < C.oc.size(); ++s) C.fidx.push_back((int)(C.own + (long long)s));
          } else {
            for (int c = 0; c < 4; ++c) {
              const ABox& ch = tree[j + 1][B.child[c]];
              const auto& v = (j == level_LFR - 1 || ch.leaf) ? ch.lfr.fidx : ch.cones[cone / 2].fidx;
              C.fidx.insert(C.fidx.end(), v.begin(), v.end());
            }
          }
        }
      }
    }
  // ---- potentials P: leaf points, then every non-leaf node with user checks.
  long long P = N;
  for (int j = 2; j <= nLevels; ++j)
    for (int k = 0; k < (int)tree[j].size(); ++k) {
      ABox& B = tree[j][k];
      if (B.leaf) continue;
      if (j >= level_LFR) {
        if (!B.lfr.uc.empty()) { B.lfr.pot = P; P += (long long)B.lfr.uc.size(); }
      } else {
        for (ANode& C : B.cones)
          if (!C.uc.empty()) { C.pot = P; P += (long long)C.uc.size(); }
      }
    }
  op.charges_len = S;
  op.pots_len = P;
  auto pot_of = [&](int j, int k, int cone) -> long long {  // first potential row of a node
    const ABox& B = tree[j][k];
    if (B.leaf) return B.pt0;
    return cone < 0 ? B.lfr.pot : B.cones[cone].pot;
  };

  // ---- upward: T = Atilde^{-1} Ar (LFR boxes and leaves) or Atilde^{-1} M2M (cones).
  op.up.clear();
  for (int j = nLevels; j >= 2; --j) {
    std::vector<std::pair<int, int>> work;
    for (int k = 0; k < (int)tree[j].size(); ++k) {
      if (lfr_box(j, k)) work.push_back({k, -1});
      else for (int c = 0; c < nCones[j]; ++c) work.push_back({k, c});
    }
    std::vector<std::vector<cd>> T(work.size());
    std::vector<std::vector<int>> src(work.size());
#pragma omp parallel for schedule(dynamic, 1)
    for (int t = 0; t < (int)work.size(); ++t) {
      const int k = work[t].first, cone = work[t].second;
      ABox& B = tree[j][k];
      ANode& nd = cone < 0 ? B.lfr : B.cones[cone];
      if (!nd.out_active || nd.oc.empty()) continue;
      HCache hc{this, {}};
      std::vector<int> s, spts;
      if (B.leaf) {
        for (int i = 0; i < rank; ++i) s.push_back(B.pt0 + i);
        spts = s;
      } else {
        for (int c = 0; c < 4; ++c) {
          const ABox& ch = tree[j + 1][B.child[c]];
          const ANode& cn = (cone < 0 || j == level_LFR - 1 || ch.leaf) ? ch.lfr : ch.cones[cone / 2];
          s.insert(s.end(), cn.fidx.begin(), cn.fidx.end());
          spts.insert(spts.end(), cn.oc.begin(), cn.oc.end());
        }
      }
      const int r = (int)nd.oc.size(), K = (int)s.size();
      if (K == 0 || nd.ochk.empty()) continue;
      // LFR: the ACA's pivot rows; cones: M2M = K(check points, children's charge points).
      const std::vector<cd> Arow = cone < 0 ? nd.Ar : block(nd.ochk, spts, hc);
      std::vector<cd> At((size_t)r * r);  // Atilde = K(ochk, oc), column major
      {
        const std::vector<cd> A = block(nd.ochk, nd.oc, hc);
        for (int a = 0; a < r; ++a)
          for (int c = 0; c < r; ++c) At[(size_t)c * r + a] = A[(size_t)a * r + c];
      }
      PivQR qr;
      qr.factor(r, r, At);
      std::vector<cd> Tm((size_t)r * K), col(r), sol(r);
      for (int c = 0; c < K; ++c) {
        for (int a = 0; a < r; ++a) col[a] = Arow[(size_t)a * K + c];
        qr.solve(col.data(), sol.data());
        for (int a = 0; a < r; ++a) Tm[(size_t)a * K + c] = sol[a];
      }
      T[t] = std::move(Tm);
      src[t] = std::move(s);
    }
    GemvPhase ph;
    stage_blocks(ph, (int)work.size(), [&](int t) {
      if (T[t].empty()) return BlockView{nullptr, 0, 0, nullptr, 0};
      const ABox& B = tree[j][work[t].first];
      const ANode& nd = work[t].second < 0 ? B.lfr : B.cones[work[t].second];
      return BlockView{&T[t], (int)nd.oc.size(), (int)src[t].size(), &src[t], (int)nd.own};
    });
    finalize(ph, "UP");
    op.up.push_back(std::move(ph));
  }

  // ---- M2L: LFR boxes (leaves on any level) and HFR cones with interaction lists.
  {
    struct Task { std::vector<cd> A; std::vector<int> idx; int rows = 0, K = 0; long long out = 0; };
    std::vector<std::tuple<int, int, int>> all;
    for (int j = 2; j <= nLevels; ++j)
      for (int k = 0; k < (int)tree[j].size(); ++k) {
        if (lfr_box(j, k)) all.push_back({j, k, -1});
        else for (int c = 0; c < nCones[j]; ++c) all.push_back({j, k, c});
      }
    std::vector<Task> tasks(all.size());
#pragma omp parallel for schedule(dynamic, 1)
    for (int u = 0; u < (int)all.size(); ++u) {
      const int j = std::get<0>(all[u]), k = std::get<1>(all[u]), cone = std::get<2>(all[u]);
      ABox& B = tree[j][k];
      ANode& nd = cone < 0 ? B.lfr : B.cones[cone];
      if (!nd.in_active || nd.uc.empty()) continue;
      std::vector<const ANode*> srcs;
      for (const Ref& p : nd.IL) {
        const ABox& O = box(p);
        const ANode& s = (cone >= 0 && O.leaf) ? O.lfr : partner(p, j, k);
        if (!s.oc.empty()) srcs.push_back(&s);
      }
      int K = 0;
      for (const ANode* s : srcs) K += (int)s->oc.size();
      if (K == 0) continue;
      HCache hc{this, {}};
      Task& tk = tasks[u];
      const int rows = (int)nd.uc.size();
      tk.A.assign((size_t)rows * K, cd(0.0, 0.0));
      int c0 = 0;
      for (const ANode* s : srcs) {
        const std::vector<cd> blk = block(nd.uc, s->oc, hc);
        const int w = (int)s->oc.size();
        for (int a = 0; a < rows; ++a)
          for (int c = 0; c < w; ++c) tk.A[(size_t)a * K + c0 + c] = blk[(size_t)a * w + c];
        tk.idx.insert(tk.idx.end(), s->fidx.begin(), s->fidx.end());
        c0 += w;
      }
      tk.rows = rows;
      tk.K = K;
      tk.out = pot_of(j, k, cone);
    }
    GemvPhase ph;
    op.m2l_rows = 0;
    for (auto& tk : tasks)
      if (tk.K != 0) op.m2l_rows += tk.rows;
    stage_blocks(ph, (int)tasks.size(), [&](int u) {
      Task& tk = tasks[u];
      if (tk.K == 0) return BlockView{nullptr, 0, 0, nullptr, 0};
      return BlockView{&tk.A, tk.rows, tk.K, &tk.idx, (int)tk.out};
    });
    finalize(ph, "M2L");
    op.m2l = std::move(ph);
  }

  // ---- downward, parents at level j to children at j + 1 (HFR_L2L :4208 for
  // HFR parents, LFR_L2L :2800 for LFR parents).
  op.down.clear();
  for (int j = 2; j < nLevels; ++j) {
    // QR of Atilde_in^T of every IL-active parent node with incoming charges.
    std::vector<std::tuple<int, int>> parents;
    for (int k = 0; k < (int)tree[j].size(); ++k) {
      if (tree[j][k].leaf) continue;
      if (j >= level_LFR) parents.push_back({k, -1});
      else for (int c = 0; c < nCones[j]; ++c) parents.push_back({k, c});
    }
    std::map<std::pair<int, int>, PivQR> AT;
    for (auto& p : parents) AT[{std::get<0>(p), std::get<1>(p)}] = PivQR();
    std::vector<std::pair<int, int>> keys;
    for (auto& kv : AT) keys.push_back(kv.first);
#pragma omp parallel for schedule(dynamic, 1)
    for (int t = 0; t < (int)keys.size(); ++t) {
      const int k = keys[t].first, cone = keys[t].second;
      const ANode& p = cone < 0 ? tree[j][k].lfr : tree[j][k].cones[cone];
      if (!p.in_active || p.ic.empty() || p.pot < 0) continue;
      HCache hc{this, {}};
      const int r = (int)p.ic.size();
      const std::vector<cd> A = block(p.ichk, p.ic, hc);  // row major r x r
      // A row major is A^T column major: the matrix W = Lb A^{-1} needs.
      AT[keys[t]].factor(r, r, A);
    }
    // Child nodes at level j + 1 and the parent terms that feed them.
    struct Child { int k, cone; };  // cone < 0: the box's LFR node (or a leaf)
    std::vector<Child> kids;
    for (int k = 0; k < (int)tree[j].size(); ++k) {
      const ABox& B = tree[j][k];
      if (B.leaf) continue;
      for (int c = 0; c < 4; ++c) {
        const int kc = B.child[c];
        const ABox& ch = tree[j + 1][kc];
        if (j + 1 >= level_LFR || ch.leaf) kids.push_back({kc, -1});
        else for (int cc = 0; cc < nCones[j + 1]; ++cc) kids.push_back({kc, cc});
      }
    }
    // parent index of every box at level j + 1
    std::vector<int> parent(tree[j + 1].size(), -1), slot(tree[j + 1].size(), -1);
    for (int k = 0; k < (int)tree[j].size(); ++k)
      for (int c = 0; c < 4; ++c)
        if (tree[j][k].child[c] >= 0) { parent[tree[j][k].child[c]] = k; slot[tree[j][k].child[c]] = c; }
    // Length of child c's rows inside a pass-through parent potential.
    auto child_len = [&](int kp, int c, int pcone) -> int {
      const ABox& ch = tree[j + 1][tree[j][kp].child[c]];
      if (pcone < 0 || j == level_LFR - 1) return ch.leaf ? rank : (int)ch.lfr.uc.size();
      return ch.leaf ? (int)ch.lfr.uc.size() : (int)ch.cones[pcone / 2].uc.size();
    };
    struct Task { std::vector<cd> A; std::vector<int> idx; int rows = 0, K = 0; long long out = 0; bool any = false; };
    std::vector<Task> tasks(kids.size());
#pragma omp parallel for schedule(dynamic, 1)
    for (int t = 0; t < (int)kids.size(); ++t) {
      const int kc = kids[t].k, cc = kids[t].cone;
      const ABox& X = tree[j + 1][kc];
      const ANode& xn = cc < 0 ? X.lfr : X.cones[cc];
      const std::vector<int> rows_pts = X.leaf ? xn.uc : xn.uc;
      const int rows = (int)rows_pts.size();
      if (rows == 0) continue;
      const int kp = parent[kc], child = slot[kc];
      std::vector<int> pcones;
      if (j >= level_LFR) pcones.push_back(-1);
      else for (int pc = 0; pc < nCones[j]; ++pc) if (cc < 0 || pc / 2 == cc) pcones.push_back(pc);
      HCache hc{this, {}};
      Task& tk = tasks[t];
      std::vector<std::vector<cd>> cols_blocks;
      std::vector<int> widths;
      for (int pc : pcones) {
        const ANode& p = pc < 0 ? tree[j][kp].lfr : tree[j][kp].cones[pc];
        if (p.pot < 0) continue;
        if (p.in_active) {
          if (p.ic.empty()) continue;
          const int r = (int)p.ic.size();
          const std::vector<cd> Lb = block(rows_pts, p.ic, hc);
          std::vector<cd> W;
          fold_right_inverse(Lb, rows, r, AT.at({kp, pc}), W);
          cols_blocks.push_back(std::move(W));
          widths.push_back(r);
          for (int m = 0; m < r; ++m) tk.idx.push_back((int)(p.pot + m));
        } else {
          int off = 0;
          for (int c = 0; c < child; ++c) off += child_len(kp, c, pc);
          std::vector<cd> Id((size_t)rows * rows, cd(0.0, 0.0));
          for (int a = 0; a < rows; ++a) Id[(size_t)a * rows + a] = 1.0;
          cols_blocks.push_back(std::move(Id));
          widths.push_back(rows);
          for (int m = 0; m < rows; ++m) tk.idx.push_back((int)(p.pot + off + m));
        }
      }
      int K = 0;
      for (int w : widths) K += w;
      if (K == 0) continue;
      tk.A.assign((size_t)rows * K, cd(0.0, 0.0));
      int c0 = 0;
      for (size_t b = 0; b < cols_blocks.size(); ++b) {
        for (int a = 0; a < rows; ++a)
          for (int c = 0; c < widths[b]; ++c) tk.A[(size_t)a * K + c0 + c] = cols_blocks[b][(size_t)a * widths[b] + c];
        c0 += widths[b];
      }
      tk.rows = rows;
      tk.K = K;
      tk.out = X.leaf ? X.pt0 : xn.pot;
      tk.any = tk.out >= 0;
    }
    GemvPhase ph;
    ph.accumulate = 1;
    stage_blocks(ph, (int)tasks.size(), [&](int t) {
      Task& tk = tasks[t];
      if (!tk.any) return BlockView{nullptr, 0, 0, nullptr, 0};
      return BlockView{&tk.A, tk.rows, tk.K, &tk.idx, (int)tk.out};
    });
    finalize(ph, "DOWN");
    op.down.push_back(std::move(ph));
  }

  // ---- near field (evaluate_NearField_Using_Precomputations_LS :2884-2960):
  // per leaf, diag(kappa^2 q) B (+ I for the self block) of every
  // neighbour, accumulated into the leaf's potentials.
  {
    const int nl = (int)leaves.size();
    std::vector<std::vector<cd>> A(nl);
    std::vector<std::vector<int>> idx(nl);
#pragma omp parallel for schedule(dynamic, 4)
    for (int t = 0; t < nl; ++t) {
      const ABox& B = box(leaves[t]);
      const int j = leaves[t].first;
      std::vector<std::pair<const std::vector<cd>*, int>> terms;  // block, source first point
      for (int kind = 0; kind < 4; ++kind)
        for (int n = 0; n < kNbrCount[kind]; ++n) {
          const int nk = B.nbr[kind][n];
          if (nk < 0) continue;
          terms.push_back({&nearBlk.at(std::make_tuple(j, kind, n)), tree[j + kNbrLevel[kind]][nk].pt0});
        }
      const int K = (int)terms.size() * rank;
      std::vector<cd>& a = A[t];
      a.assign((size_t)rank * K, cd(0.0, 0.0));
      for (size_t q = 0; q < terms.size(); ++q) {
        const std::vector<cd>& Bk = *terms[q].first;
        const bool self = terms[q].second == B.pt0;
        for (int i = 0; i < rank; ++i) {
          const double s = cfg.findPhi ? kq[B.pt0 + i] : 1.0;
          for (int c = 0; c < rank; ++c) {
            cd v = s * Bk[(size_t)i * rank + c];
            if (cfg.findPhi && self && i == c) v += 1.0;
            a[(size_t)i * K + q * rank + c] = v;
          }
        }
        for (int c = 0; c < rank; ++c) idx[t].push_back(terms[q].second + c);
      }
    }
    GemvPhase ph;
    ph.accumulate = 1;
    stage_blocks(ph, nl, [&](int t) {
      return BlockView{&A[t], rank, (int)idx[t].size(), &idx[t], box(leaves[t]).pt0};
    });
    finalize(ph, "DOWN");
    op.nearph = std::move(ph);
    op.generic_near = true;
  }
}

bool AdaptiveBuilder::run(HostOperator& op, std::string& err) {
  const auto t0 = std::chrono::steady_clock::now();
  if (cfg.nChebNodes < 2 || cfg.nChebNodes > 8) { err = "nChebNodes must be in [2, 8]"; return false; }
  if (cfg.degreeOfBases < 1 || cfg.degreeOfBases * (cfg.degreeOfBases + 1) / 2 > cfg.nChebNodes * cfg.nChebNodes) {
    err = "degreeOfBases gives more basis polynomials than nodes"; return false;
  }
  if (!(cfg.L > 0.0) || !(cfg.kappa >= 0.0)) { err = "L must be > 0 and kappa >= 0"; return false; }
  if (cfg.Qchoice < 0 || cfg.Qchoice > 6) { err = "Qchoice must be in [0, 6]"; return false; }
  if (cfg.Qchoice == 6 && (cfg.n_bumps < 1 || cfg.n_bumps > LS_MAX_BUMPS)) { err = "n_bumps must be in [1, 8]"; return false; }
  if (cfg.nCones_LFR < 1 || cfg.TOL_POW < 1 || cfg.TOL_POW > 16) { err = "nCones_LFR >= 1 and TOL_POW in [1, 16] required"; return false; }
  if (cfg.treeAdaptivity < 1 || cfg.treeAdaptivity > 12) { err = "treeAdaptivity must be in [1, 12]"; return false; }
  auto lap = [t = t0]() mutable {
    const auto now = std::chrono::steady_clock::now();
    const double s = std::chrono::duration<double>(now - t).count();
    t = now;
    return s;
  };
  kappa = cfg.kappa;
  L = cfg.L;
  n1 = cfg.nChebNodes;
  rank = n1 * n1;
  nb = cfg.degreeOfBases * (cfg.degreeOfBases + 1) / 2;
  epsTree = std::pow(10, -cfg.treeAdaptivity);
  if (cfg.yes2DFMM == 1) {
    level_LFR = kappa == 0 ? 2 : (int)std::floor(std::log(kappa * L / 0.35) / std::log(2.0));
    if (level_LFR < 2) level_LFR = 2;
  } else {
    level_LFR = 2;
  }
  cheb_setup();
  for (int d = 0; d < cfg.degreeOfBases; ++d)
    for (int a = 0; a < d + 1; ++a) bases.push_back({a, d - a});
  tree.assign(1, {});
  ABox root;
  root.r = L;
  tree[0].push_back(root);
  create_tree(0, 0);
  nLevels = (int)tree.size() - 1;
  if (nLevels < 3 || nLevels > 12) { err = "the adaptive tree has " + std::to_string(nLevels) + " levels (3..12 supported)"; return false; }
  radius.push_back(L);
  for (int j = 1; j <= std::max(10, nLevels + 1); ++j) radius.push_back(radius[j - 1] / 2.0);
  if (level_LFR >= nLevels) level_LFR = nLevels - 1;
  level_restriction();
  nCones.push_back((int)(cfg.nCones_LFR * std::pow(2.0, level_LFR - 1)));
  aperture.push_back(2 * kPi / nCones[0]);
  for (int j = 1; j <= level_LFR - 1; ++j) {
    nCones.push_back((int)(nCones[j - 1] / 2.0));
    aperture.push_back(aperture[j - 1] * 2.0);
  }
  for (int j = 0; j <= level_LFR - 1 && j <= nLevels; ++j)
    for (auto& B : tree[j])
      if (!B.leaf) B.cones.assign(nCones[j], ANode());
  for (int c = 0; c < 4; ++c)
    for (int n = 0; n < 4; ++n) tree[1][c].nbrs.push_back({1, n});
  for (int j = 1; j <= nLevels - 1; ++j)
    for (int k = 0; k < (int)tree[j].size(); ++k)
      if (!tree[j][k].leaf)
        for (int c = 0; c < 4; ++c) child_interactions(c, j, k);
  // points (assignLeafChargeLocations :1150-1163)
  for (size_t t = 0; t < leaves.size(); ++t) {
    ABox& B = box(leaves[t]);
    B.pt0 = N;
    for (int i = 0; i < rank; ++i) {
      gx.push_back(radius[leaves[t].first] * cheb1[i % n1] + B.cx);
      gy.push_back(radius[leaves[t].first] * cheb1[i / n1] + B.cy);
      leaf_of.push_back((int)t);
    }
    N += rank;
  }
  kq.resize(N);
  for (int i = 0; i < N; ++i) kq[i] = kappa * kappa * (contrast(gx[i], gy[i]));
  op.stage_seconds[0] = lap();
  gl_rule(kQuadOrder, gln, glw);
  precompute_Q();
  std::set<int> leaf_levels;
  for (const Ref& lf : leaves) leaf_levels.insert(lf.first);
  classify_neighbors();
  if (unmatched) { err = "adaptive tree: " + std::to_string(unmatched) + " near neighbours of unexpected level or offset"; return false; }
  precomputations(leaf_levels);
  op.stage_seconds[1] = lap();
  op.stage_seconds[2] = lap();
  nca();
  op.stage_seconds[3] = lap();
  user_checks();
  op.stage_seconds[4] = lap();
  pack(op);
  op.stage_seconds[5] = lap();
  op.cfg = cfg;
  op.N = N;
  op.n_leaves = (int)leaves.size();
  op.rank = rank;
  op.n_levels = nLevels;
  op.level_LFR = level_LFR;
  op.n_bases = nb;
  op.px = gx;
  op.py = gy;
  op.q.resize(N);
  for (int i = 0; i < N; ++i) op.q[i] = contrast(gx[i], gy[i]);
  op.kq = kq;
  op.Qpinv = Qp;
  op.M.assign((size_t)rank * (2 * kSeries + 1), cd());
  {
    const std::vector<cd>& Mf = Mlev.rbegin()->second;  // finest leaf level
    for (size_t i = 0; i < op.M.size(); ++i) op.M[i] = Mf[i];
  }
  // Skeleton dump: per box of levels 2..nLevels (per cone for non-leaf HFR
  // boxes, cone -1 otherwise) j, k, cone, then the outgoing charge,
  // outgoing check, incoming charge and incoming check point lists, each
  // as a length and the point indices.
  op.skeleton_dump.clear();
  int mr = 0;
  auto put = [&](int v) { op.skeleton_dump.push_back(v); };
  auto putv = [&](const std::vector<int>& v) { put((int)v.size()); for (int x : v) put(x); };
  for (int j = 2; j <= nLevels; ++j)
    for (int k = 0; k < (int)tree[j].size(); ++k) {
      const ABox& B = tree[j][k];
      auto rec = [&](const ANode& nd, int cone) {
        put(j); put(k); put(cone);
        putv(nd.oc); putv(nd.ochk); putv(nd.ic); putv(nd.ichk);
        if (nd.out_active) mr = std::max(mr, (int)nd.oc.size());
        if (nd.in_active) mr = std::max(mr, (int)nd.ic.size());
      };
      if (lfr_box(j, k)) rec(B.lfr, -1);
      else for (int c = 0; c < (int)B.cones.size(); ++c) rec(B.cones[c], c);
    }
  op.max_rank = mr;
  op.assemble_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return true;
}
