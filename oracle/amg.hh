// ORACLE -- test infrastructure only (included by oracle.cc).
//
// Restatement of the algebraic multigrid preconditioner of the reference's
// ParallelAmgBackend (opm/simulators/linalg/parallelamgbackend.hh:85-330):
// BiCGStab (the same BiCGStabSolver as the ILU(0) backend) preconditioned by
// one V-cycle of an aggregation AMG built from the system matrix.
//
// The reference hands the matrix to dune-istl's Dune::Amg::AMG, which is not
// vendored; its published structure is restated here with the parameters the
// backend sets (parallelamgbackend.hh:262-305):
//   * coarsening stops at AmgCoarsenTarget (5000) rows, at 15 levels, or when
//     a level shrinks by less than the minimum coarsen rate 1.05;
//   * strength of connection on the Frobenius norms of the blocks
//     (SymmetricCriterion<FrobeniusNorm>), threshold alpha = 1/3;
//   * piecewise-constant prolongation over aggregates, damped by 1.6; the
//     coarse matrix is the Galerkin product P^T A P;
//   * one SOR step (relaxation 1.0) per smoothing step, 2 pre- and 2
//     post-smoothing steps, forward before and backward after the coarse
//     correction; V-cycle (gamma 1), zero initial guess.
// Where the GPU form deviates from dune-istl (each deviation is the same in
// the GPU code and here, so the two agree):
//   * aggregation: Vanek-Mandel-Brezina greedy aggregation (a root and its
//     strong neighbours; left-over rows join the strongest neighbouring
//     aggregate; the rest form aggregates of their own) instead of dune's
//     diameter-bounded aggregate growing;
//   * the SOR sweeps visit the rows colour by colour (greedy colouring of the
//     level's graph, in row order on the finest level and in smallest-last
//     order on the coarse ones), rows of one colour in any order -- the
//     natural-order sweep of dune-istl is one chain of dependent rows;
//   * the coarsest level is smoothed (2 forward + backward sweep pairs)
//     instead of being solved directly;
//   * aggregates, colours and coarse patterns are built from the first
//     matrix a solver sees and kept for later matrices of the same pattern
//     (the reference rebuilds the hierarchy at every solve); the coarse
//     values and the inverted diagonals are recomputed at every solve.
// Operation orders (so that the GPU's FP64 results can be compared with
// these bit for bit where no reduction is involved):
//   * Galerkin sum: coarse row I's members in ascending row order, each
//     member's entries in ascending column order, added into the coarse
//     block of the entry's aggregate starting from 0;
//   * restriction: the members' defects in ascending row order from 0;
//   * a row's smoothing update: v = rhs_i; v -= A_ij x_j (j != i, ascending
//     columns, mmv order); x_i = D_i^-1 v (row-major, sums from 0);
//   * the defect: rhs_i - (sum over columns of A_ij x_j, spmv order);
//   * prolongation: x_i += 1.6 * x_c.
// Included inside namespace oracle after the block helpers (<algorithm> and
// <functional> come from oracle.cc).
struct AmgLevel {
    Bcrs A;                          // this level's matrix (natural row order of the level)
    std::vector<int> color;          // colour of each row
    std::vector<int> colorPtr;       // rows of colour c: colorRows[colorPtr[c] .. colorPtr[c + 1])
    std::vector<int> colorRows;      // ascending within a colour
    std::vector<double> dinv;        // inverted diagonal blocks, n * b * b
    std::vector<int> agg;            // row -> row of the next level (all levels but the coarsest)
    int nextN = 0;
    // Galerkin map to the next level: for coarse block k, the fine blocks
    // gIdx[gPtr[k] .. gPtr[k + 1]) summed in that order
    std::vector<int> gPtr, gIdx;
};

struct AmgHierarchy {
    std::vector<AmgLevel> lv;
    bool built = false;
};

constexpr int AMG_MAX_LEVELS = 15;
constexpr double AMG_MIN_COARSEN_RATE = 1.05;
constexpr double AMG_ALPHA = 1.0 / 3.0;
constexpr double AMG_PROLONG_DAMP = 1.6;
constexpr int AMG_PRE_SMOOTH = 2;
constexpr int AMG_POST_SMOOTH = 2;
constexpr int AMG_COARSEST_PAIRS = 2;

static double frobenius(const double* blk, int bb)
{
    double s = 0;
    for (int e = 0; e < bb; ++e) s += blk[e] * blk[e];
    return std::sqrt(s);
}

// strong neighbours of every row (ascending), from the block norms: (i, j)
// is strong when |A_ij| >= alpha * max_k!=i |A_ik| or |A_ji| >= alpha *
// max_k!=j |A_jk| (the symmetric criterion)
static std::vector<std::vector<int>> strongGraph(const Bcrs& A, std::vector<double>& nrm)
{
    const int n = A.n, bb = A.b * A.b;
    nrm.assign(A.col.size(), 0.0);
    std::vector<double> mx(n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int k = A.rowPtr[i]; k < A.rowPtr[i + 1]; ++k) {
            nrm[k] = frobenius(&A.val[(size_t)k * bb], bb);
            if (A.col[k] != i) mx[i] = std::max(mx[i], nrm[k]);
        }
    std::vector<std::vector<int>> S(n);
    for (int i = 0; i < n; ++i)
        for (int k = A.rowPtr[i]; k < A.rowPtr[i + 1]; ++k) {
            const int j = A.col[k];
            if (j == i) continue;
            const int kt = A.find(j, i);
            const bool si = mx[i] > 0 && nrm[k] >= AMG_ALPHA * mx[i];
            const bool sj = kt >= 0 && mx[j] > 0 && nrm[kt] >= AMG_ALPHA * mx[j];
            if (si || sj) S[i].push_back(j);
        }
    return S;
}

// greedy aggregation (Vanek, Mandel, Brezina 1996): returns the number of
// aggregates, agg[i] = aggregate of row i, numbered in creation order
static int aggregate(const Bcrs& A, std::vector<int>& agg)
{
    const int n = A.n;
    std::vector<double> nrm;
    const std::vector<std::vector<int>> S = strongGraph(A, nrm);
    agg.assign(n, -1);
    int na = 0;
    // 1: a row whose strong neighbours are all free roots an aggregate of them
    for (int i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        bool free = true;
        for (int j : S[i]) free = free && agg[j] < 0;
        if (!free) continue;
        agg[i] = na;
        for (int j : S[i]) agg[j] = na;
        ++na;
    }
    // 2: a free row joins the aggregate (from step 1) of its strongest
    // strong neighbour; ties go to the lowest column
    const std::vector<int> agg1 = agg;
    for (int i = 0; i < n; ++i) {
        if (agg1[i] >= 0) continue;
        double best = -1;
        int pick = -1;
        for (int k = A.rowPtr[i]; k < A.rowPtr[i + 1]; ++k) {
            const int j = A.col[k];
            if (j == i || agg1[j] < 0) continue;
            if (!std::binary_search(S[i].begin(), S[i].end(), j)) continue;
            const int kt = A.find(j, i);
            const double s = std::max(nrm[k], kt >= 0 ? nrm[kt] : 0.0);
            if (s > best) { best = s; pick = agg1[j]; }
        }
        if (pick >= 0) agg[i] = pick;
    }
    // 3: the rows still free root aggregates of themselves and their free
    // strong neighbours
    for (int i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        agg[i] = na;
        for (int j : S[i])
            if (agg[j] < 0) agg[j] = na;
        ++na;
    }
    return na;
}

// pattern of the Galerkin product and the map of fine blocks per coarse block
static void galerkinPattern(const Bcrs& A, const std::vector<int>& agg, int nc, Bcrs& Ac, std::vector<int>& gPtr,
                            std::vector<int>& gIdx)
{
    std::vector<std::vector<int>> members(nc);
    for (int i = 0; i < A.n; ++i) members[agg[i]].push_back(i);
    Ac.n = nc;
    Ac.b = A.b;
    Ac.rowPtr.assign(nc + 1, 0);
    Ac.col.clear();
    for (int I = 0; I < nc; ++I) {
        std::vector<int> cols;
        for (int i : members[I])
            for (int k = A.rowPtr[i]; k < A.rowPtr[i + 1]; ++k) cols.push_back(agg[A.col[k]]);
        std::sort(cols.begin(), cols.end());
        cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
        Ac.col.insert(Ac.col.end(), cols.begin(), cols.end());
        Ac.rowPtr[I + 1] = (int)Ac.col.size();
    }
    const int nnzc = Ac.rowPtr[nc];
    std::vector<std::vector<int>> lists(nnzc);
    for (int I = 0; I < nc; ++I)
        for (int i : members[I])
            for (int k = A.rowPtr[i]; k < A.rowPtr[i + 1]; ++k) lists[Ac.find(I, agg[A.col[k]])].push_back(k);
    gPtr.assign(nnzc + 1, 0);
    gIdx.clear();
    for (int k = 0; k < nnzc; ++k) {
        gIdx.insert(gIdx.end(), lists[k].begin(), lists[k].end());
        gPtr[k + 1] = (int)gIdx.size();
    }
    Ac.val.assign((size_t)nnzc * A.b * A.b, 0.0);
}

static void galerkinValues(const Bcrs& A, const std::vector<int>& gPtr, const std::vector<int>& gIdx, Bcrs& Ac)
{
    const int bb = A.b * A.b;
    for (size_t k = 0; k + 1 < gPtr.size(); ++k)
        for (int e = 0; e < bb; ++e) {
            double s = 0.0;
            for (int q = gPtr[k]; q < gPtr[k + 1]; ++q) s += A.val[(size_t)gIdx[q] * bb + e];
            Ac.val[k * bb + e] = s;
        }
}

// smallest-last vertex order (Matula and Beck 1983): repeatedly remove the
// row of least degree among those left (ties: the lowest row); the colouring
// visits them in the reverse order of removal
static std::vector<int> smallestLastOrder(const Bcrs& A)
{
    const int n = A.n;
    std::vector<int> deg(n, 0);
    for (int i = 0; i < n; ++i)
        for (int k = A.rowPtr[i]; k < A.rowPtr[i + 1]; ++k)
            if (A.col[k] != i) ++deg[i];
    std::set<std::pair<int, int>> left;
    for (int i = 0; i < n; ++i) left.insert({deg[i], i});
    std::vector<char> gone(n, 0);
    std::vector<int> order;
    order.reserve(n);
    while (!left.empty()) {
        const int v = left.begin()->second;
        left.erase(left.begin());
        gone[v] = 1;
        order.push_back(v);
        for (int k = A.rowPtr[v]; k < A.rowPtr[v + 1]; ++k) {
            const int j = A.col[k];
            if (j == v || gone[j]) continue;
            left.erase({deg[j], j});
            --deg[j];
            left.insert({deg[j], j});
        }
    }
    std::reverse(order.begin(), order.end());
    return order;
}

// greedy colouring: the smallest colour no coloured neighbour has, the rows
// visited in row order on the finest level (a red-black colouring of the
// 5/7-point pattern) and in smallest-last order on the coarse levels
// (fewer colours on the aggregates' graphs)
static void colour(AmgLevel& L, bool finest)
{
    const Bcrs& A = L.A;
    L.color.assign(A.n, -1);
    int nc = 0;
    std::vector<int> seen;
    std::vector<int> order;
    if (!finest) order = smallestLastOrder(A);
    for (int t = 0; t < A.n; ++t) {
        const int i = finest ? t : order[t];
        seen.assign(nc + 1, 0);
        for (int k = A.rowPtr[i]; k < A.rowPtr[i + 1]; ++k) {
            const int j = A.col[k];
            if (j != i && L.color[j] >= 0) seen[L.color[j]] = 1;
        }
        int c = 0;
        while (seen[c]) ++c;
        L.color[i] = c;
        nc = std::max(nc, c + 1);
    }
    L.colorPtr.assign(nc + 1, 0);
    for (int i = 0; i < A.n; ++i) L.colorPtr[L.color[i] + 1]++;
    for (int c = 0; c < nc; ++c) L.colorPtr[c + 1] += L.colorPtr[c];
    L.colorRows.assign(A.n, 0);
    std::vector<int> pos(L.colorPtr.begin(), L.colorPtr.end() - 1);
    for (int i = 0; i < A.n; ++i) L.colorRows[pos[L.color[i]]++] = i;
}

static void invertDiagonals(AmgLevel& L)
{
    const Bcrs& A = L.A;
    const int bb = A.b * A.b;
    L.dinv.assign((size_t)A.n * bb, 0.0);
    for (int i = 0; i < A.n; ++i) {
        const int k = A.find(i, i);
        if (k < 0) throw NumericalProblem("diagonal entry missing", GBFV_ERR_ARG);
        std::memcpy(&L.dinv[(size_t)i * bb], &A.val[(size_t)k * bb], sizeof(double) * bb);
        blockInvert(A.b, &L.dinv[(size_t)i * bb]);
    }
}

// AMG::AMG(...) with the backend's coarsening criterion: the hierarchy's
// structure from A's values (first call), the values of every level (each call)
static void amgSetup(AmgHierarchy& H, const Bcrs& A, int coarsenTarget)
{
    if (!H.built) {
        H.lv.clear();
        H.lv.emplace_back();
        H.lv[0].A = A;
        while ((int)H.lv.size() < AMG_MAX_LEVELS && H.lv.back().A.n > coarsenTarget) {
            AmgLevel& L = H.lv.back();
            std::vector<int> agg;
            const int nc = aggregate(L.A, agg);
            if ((double)L.A.n / nc < AMG_MIN_COARSEN_RATE) break;
            AmgLevel next;
            galerkinPattern(L.A, agg, nc, next.A, L.gPtr, L.gIdx);
            galerkinValues(L.A, L.gPtr, L.gIdx, next.A);
            L.agg = agg;
            L.nextN = nc;
            H.lv.push_back(std::move(next));
        }
        for (size_t l = 0; l < H.lv.size(); ++l) colour(H.lv[l], l == 0);
        H.built = true;
    }
    else {
        H.lv[0].A.val = A.val;
        for (size_t l = 0; l + 1 < H.lv.size(); ++l) galerkinValues(H.lv[l].A, H.lv[l].gPtr, H.lv[l].gIdx, H.lv[l + 1].A);
    }
    for (AmgLevel& L : H.lv) invertDiagonals(L);
}

// one SOR sweep (relaxation 1) colour by colour, forward or backward; with
// `fromZero` the rows not yet visited in this sweep count as zero (the first
// sweep of a zero initial guess)
static void sorSweep(const AmgLevel& L, std::vector<double>& x, const std::vector<double>& rhs, bool forward,
                     bool fromZero)
{
    const Bcrs& A = L.A;
    const int b = A.b, bb = b * b, nc = (int)L.colorPtr.size() - 1;
    for (int q = 0; q < nc; ++q) {
        const int c = forward ? q : nc - 1 - q;
        for (int p = L.colorPtr[c]; p < L.colorPtr[c + 1]; ++p) {
            const int i = L.colorRows[p];
            double v[3];
            for (int e = 0; e < b; ++e) v[e] = rhs[(size_t)i * b + e];
            for (int k = A.rowPtr[i]; k < A.rowPtr[i + 1]; ++k) {
                const int j = A.col[k];
                if (j == i) continue;
                if (fromZero && L.color[j] >= c) continue;  // not visited yet: zero
                mmv(b, &A.val[(size_t)k * bb], &x[(size_t)j * b], v);
            }
            const double* Di = &L.dinv[(size_t)i * bb];
            for (int r = 0; r < b; ++r) {
                double s = 0;
                for (int cc = 0; cc < b; ++cc) s += Di[r * b + cc] * v[cc];
                x[(size_t)i * b + r] = s;
            }
        }
    }
}

// AMG::mgc with gamma = 1 from a zero initial guess on level l
static void vcycle(const AmgHierarchy& H, size_t l, std::vector<double>& x, const std::vector<double>& rhs)
{
    const AmgLevel& L = H.lv[l];
    const int b = L.A.b, bb = b * b, n = L.A.n;
    x.assign((size_t)n * b, 0.0);
    if (l + 1 == H.lv.size()) {
        for (int s = 0; s < AMG_COARSEST_PAIRS; ++s) {
            sorSweep(L, x, rhs, true, s == 0);
            sorSweep(L, x, rhs, false, false);
        }
        return;
    }
    for (int s = 0; s < AMG_PRE_SMOOTH; ++s) sorSweep(L, x, rhs, true, s == 0);
    // defect, restricted: members in ascending row order
    std::vector<double> rc((size_t)L.nextN * b, 0.0);
    for (int i = 0; i < n; ++i) {
        double y[3] = {0, 0, 0};
        for (int k = L.A.rowPtr[i]; k < L.A.rowPtr[i + 1]; ++k) {
            const double* blk = &L.A.val[(size_t)k * bb];
            const double* xj = &x[(size_t)L.A.col[k] * b];
            for (int r = 0; r < b; ++r)
                for (int c = 0; c < b; ++c) y[r] += blk[r * b + c] * xj[c];
        }
        for (int e = 0; e < b; ++e) rc[(size_t)L.agg[i] * b + e] += rhs[(size_t)i * b + e] - y[e];
    }
    std::vector<double> xc;
    vcycle(H, l + 1, xc, rc);
    for (int i = 0; i < n; ++i)
        for (int e = 0; e < b; ++e) {
            const double t = AMG_PROLONG_DAMP * xc[(size_t)L.agg[i] * b + e];
            x[(size_t)i * b + e] += t;
        }
    for (int s = 0; s < AMG_POST_SMOOTH; ++s) sorSweep(L, x, rhs, false, false);
}

// the preconditioner application v = M^-1 d
static void amgApply(const AmgHierarchy& H, std::vector<double>& v, const std::vector<double>& d)
{
    vcycle(H, 0, v, d);
}
