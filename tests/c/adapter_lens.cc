// The lens problem (tests/problems/lensproblem.hh:227-627) run through the
// reference-side adapter (include/gbfv_opm.hh) on the test shim of the
// reference's types (opm_shim.hh): the reference's time loop, its
// timeIntegration retry and its NewtonMethod::apply loop, with the
// linearizer, the linear-solver backend and the Newton hooks of the adapter.
//
//   adapter_lens describe <file>      the gbfv_problem the adapter builds from
//                                     the problem's callbacks (no GPU)
//   adapter_lens run <steps> <nan_step> <file>
//                                     <steps> time steps from dt = 250 s; at
//                                     time step <nan_step> (-1: none) one
//                                     pressure of the host solution(0) is
//                                     replaced by NaN before the step, so the
//                                     first attempt fails and the retry runs
//                                     from the old time level with dt / 2
// Output: little-endian records (see tests/test_adapter.py).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "opm_shim.hh"
#include "../../include/gbfv_opm.hh"

namespace {

struct VgParams {  // EffToAbsLawParams<RegularizedVanGenuchtenParams> accessors
    double swr, snr, alpha, n;
    double residualSaturation(int phase) const { return phase == 0 ? swr : snr; }
    double vgAlpha() const { return alpha; }
    double vgN() const { return n; }
};

struct LiquidState {  // the fields of ImmiscibleFluidState the boundary sets
    double p[2] = {0, 0}, s[2] = {0, 0}, rho[2] = {0, 0}, mu[2] = {0, 0};
    double pressure(int ph) const { return p[ph]; }
    double saturation(int ph) const { return s[ph]; }
    double density(int ph) const { return rho[ph]; }
    double viscosity(int ph) const { return mu[ph]; }
};

// LensProblem (lensproblem.hh:227-627): 6 m x 4 m, lens [1,4] x [2,3],
// SimpleH2O / DNAPL liquids, VG materials, free-flow sides, DNAPL inlet
template <class TypeTag>
class LensProblem {
    using Simulator = Opm::GetPropType<TypeTag, Opm::Properties::Simulator>;
    using Pos = Opm::FieldVector<2>;

public:
    explicit LensProblem(Simulator& sim) : sim_(sim)
    {
        Kl_[0][0] = Kl_[1][1] = 9.05e-12;
        Ko_[0][0] = Ko_[1][1] = 4.6e-10;
        gravity_[1] = -9.81;
    }
    const Pos& gravity() const { return gravity_; }
    Pos boundingBoxMax() const
    {
        Pos p;
        p[0] = sim_.gridView().len[0];
        p[1] = sim_.gridView().len[1];
        return p;
    }
    template <class Ctx>
    const Opm::FieldMatrix<2>& intrinsicPermeability(const Ctx& c, unsigned i, unsigned t) const
    {
        return isInLens_(c.pos(i, t)) ? Kl_ : Ko_;
    }
    template <class Ctx> double porosity(const Ctx&, unsigned, unsigned) const { return 0.4; }
    template <class Ctx>
    const VgParams& materialLawParams(const Ctx& c, unsigned i, unsigned t) const
    {
        return isInLens_(c.pos(i, t)) ? lensMat_ : outerMat_;
    }
    template <class Ctx> double temperature(const Ctx&, unsigned, unsigned) const { return temperature_; }
    template <class C, class Ctx> void constraints(C& c, const Ctx&, unsigned, unsigned) const { c.setActive(false); }

    // boundary (lensproblem.hh:468-537)
    template <class Values, class Ctx>
    void boundary(Values& values, const Ctx& context, unsigned spaceIdx, unsigned timeIdx) const
    {
        const auto& pos = context.pos(spaceIdx, timeIdx);
        if (onLeftBoundary_(pos) || onRightBoundary_(pos)) {
            const double densityW = 1000.0, densityN = 1460.0;
            double pw;
            const double height = boundingBoxMax()[1];
            const double depth = boundingBoxMax()[1] - pos[1];
            if (onLeftBoundary_(pos)) {
                const double alpha = (1 + 1.5 / height);
                pw = 1e5 - alpha * densityW * gravity_[1] * depth;
            }
            else
                pw = 1e5 - densityW * gravity_[1] * depth;
            LiquidState fs;
            fs.p[0] = pw;
            fs.s[0] = 1.0;
            fs.s[1] = 0.0;
            fs.rho[0] = densityW;
            fs.rho[1] = densityN;
            fs.mu[0] = 1e-3;
            fs.mu[1] = 5.7e-4;
            values.setFreeFlow(context, spaceIdx, timeIdx, fs);
        }
        else if (onInlet_(pos)) {
            Opm::FieldVector<2> massRate(0.0);
            massRate[1] = -0.04;  // contiNEqIdx, kg / (m^2 s)
            values.setMassRate(massRate);
        }
        else
            values.setNoFlow();
    }
    // initial (lensproblem.hh:549-582): S_w = 1, hydrostatic p_w
    template <class PV, class Ctx>
    void initial(PV& values, const Ctx& context, unsigned spaceIdx, unsigned timeIdx) const
    {
        const auto& pos = context.pos(spaceIdx, timeIdx);
        const double depth = boundingBoxMax()[1] - pos[1];
        values[0] = 1e5 - 1000.0 * gravity_[1] * depth;
        values[1] = 1.0;
    }
    // FvBaseProblem::timeIntegration (fvbaseproblem.hh:512-552)
    void timeIntegration()
    {
        const unsigned maxFails = 10;
        const double minTimeStepSize = 0.0;
        for (unsigned i = 0; i < maxFails; ++i) {
            if (sim_.model().update()) return;
            ++failures;
            const double dt = sim_.timeStepSize();
            double nextDt = dt / 2.0;
            if (dt < minTimeStepSize * (1 + 1e-9)) break;
            if (nextDt < minTimeStepSize) nextDt = minTimeStepSize;
            sim_.setTimeStepSize(nextDt);
        }
        throw std::runtime_error("Newton solver didn't converge");
    }
    // nextTimeStepSize (fvbaseproblem.hh:591-610) without an end time
    double nextTimeStepSize() const
    {
        return std::min(std::numeric_limits<double>::infinity(),
                        sim_.model().newtonMethod().suggestTimeStepSize(sim_.timeStepSize()));
    }
    int failures = 0;

private:
    bool isInLens_(const Pos& pos) const
    {
        const double ll[2] = {1.0, 2.0}, ur[2] = {4.0, 3.0};
        for (int i = 0; i < 2; ++i)
            if (pos[i] < ll[i] - eps_ || pos[i] > ur[i] + eps_) return false;
        return true;
    }
    bool onLeftBoundary_(const Pos& p) const { return p[0] < eps_; }
    bool onRightBoundary_(const Pos& p) const { return p[0] > boundingBoxMax()[0] - eps_; }
    bool onUpperBoundary_(const Pos& p) const { return p[1] > boundingBoxMax()[1] - eps_; }
    bool onInlet_(const Pos& p) const
    {
        const double width = boundingBoxMax()[0];
        const double lambda = (boundingBoxMax()[0] - p[0]) / width;
        return onUpperBoundary_(p) && 0.5 < lambda && lambda < 2.0 / 3.0;
    }
    Simulator& sim_;
    Opm::FieldMatrix<2> Kl_{}, Ko_{};
    Pos gravity_;
    VgParams lensMat_{0.18, 0.0, 0.00045, 7.3}, outerMat_{0.05, 0.0, 0.0037, 4.7};
    double temperature_ = 273.15 + 20;
    double eps_ = 3e-6;
};

// the offload type tag: the reference's lens type tag with the adapter's
// linearizer, backend, Newton method and boundary-rate recorder
struct LensGbfv {
    using Scalar = double;
    using GridView = Opm::StructuredGridView<2>;
    using Simulator = Opm::Simulator<LensGbfv>;
    using Problem = LensProblem<LensGbfv>;
    using Model = Opm::Model<LensGbfv>;
    using ElementContext = Opm::ElementContext<LensGbfv>;
    using BoundaryContext = Opm::BoundaryContext<LensGbfv>;
    using BoundaryRateVector = Opm::GbfvBoundaryRateVector<LensGbfv>;
    using RateVector = Opm::FieldVector<2>;
    using Constraints = Opm::Constraints<2>;
    using PrimaryVariables = Opm::FieldVector<2>;
    using SolutionVector = std::vector<PrimaryVariables>;
    using GlobalEqVector = std::vector<Opm::FieldVector<2>>;
    using Linearizer = Opm::GbfvLinearizer<LensGbfv>;
    using LinearSolverBackend = Opm::GbfvBackend<LensGbfv>;
    using NewtonMethod = Opm::GbfvNewtonMethod<LensGbfv, Opm::NewtonMethod<LensGbfv>>;
};

template <class T> void put(FILE* f, const std::vector<T>& v)
{
    const int64_t n = int64_t(v.size());
    std::fwrite(&n, sizeof(n), 1, f);
    if (n) std::fwrite(v.data(), sizeof(T), v.size(), f);
}

Opm::StructuredGridView<2> lensGrid()
{
    Opm::StructuredGridView<2> gv;
    gv.n = {{48, 32, 1}};
    gv.len = {{6.0, 4.0, 1.0}};
    return gv;
}

}  // namespace

// The TPFA linearizer's adapter, every member compiled against the same
// shim (its numerics are tested through the C ABI, tests/test_gpu_tpfa.py)
template class Opm::GbfvTpfaLinearizer<LensGbfv>;

// what the TPFA adapter refuses, on the host (no context is created)
static int tpfaRefusals()
{
    Opm::GbfvTpfaLinearizer<LensGbfv> lin;
    int refused = 0;
    try {
        lin.setContextOptions(GBFV_MODEL_IMMISCIBLE_2P, Opm::gbfvDefaultParams());
    }
    catch (const std::runtime_error&) {
        ++refused;
    }
    Opm::LinearizationType t;
    t.type = Opm::LinearizationType::pressure;
    try {
        lin.setLinearizationType(t);
    }
    catch (const std::runtime_error&) {
        ++refused;
    }
    t.type = Opm::LinearizationType::implicit;
    t.time = 3;
    lin.setLinearizationType(t);
    const bool kept = lin.getLinearizationType().time == 3;
    lin.setContextOptions(GBFV_MODEL_BLACKOIL_3P, Opm::gbfvDefaultParams());
    const bool empty = lin.getFlowsInfo().empty() && lin.getFloresInfo().empty() && lin.getVelocityInfo().empty() &&
                       lin.constraintsMap().empty();
    std::printf("tpfa refused %d kept %d empty %d\n", refused, kept ? 1 : 0, empty ? 1 : 0);
    return refused == 2 && kept && empty ? 0 : 1;
}

int main(int argc, char** argv)
{
    if (argc >= 2 && std::string(argv[1]) == "tpfa") return tpfaRefusals();
    if (argc < 3) {
        std::fprintf(stderr, "usage: adapter_lens describe <file> | run <steps> <nan_step> <file>\n");
        return 2;
    }
    Opm::Simulator<LensGbfv> sim(lensGrid());
    const std::string mode = argv[1];
    if (mode == "describe") {
        auto D = Opm::gbfvDescribe<LensGbfv>(sim, GBFV_MODEL_IMMISCIBLE_2P);
        FILE* f = std::fopen(argv[2], "wb");
        if (!f) return 3;
        put(f, D->center);
        put(f, D->volume);
        put(f, D->porosity);
        put(f, D->perm);
        put(f, D->material);
        put(f, D->matParams);
        put(f, D->connPtr);
        put(f, D->connNbr);
        put(f, D->connDir);
        put(f, D->connNormal);
        put(f, D->connCenter);
        put(f, D->connArea);
        put(f, D->bfPtr);
        put(f, D->bfNormal);
        put(f, D->bfCenter);
        put(f, D->bfArea);
        put(f, D->bfType);
        put(f, D->bfValue);
        const gbfv_problem& P = D->prob;
        put(f, std::vector<double>{P.gravity[0], P.gravity[1], P.gravity[2], P.rho[0], P.rho[1], P.mu[0], P.mu[1],
                                   P.temperature});
        std::fclose(f);
        return 0;
    }
    if (mode != "run" || argc < 5) return 2;
    const int steps = std::atoi(argv[2]), nanStep = std::atoi(argv[3]);
    gbfv_params prm;
    gbfv_default_params(&prm);
    prm.linear_tolerance = 1e-6;
    auto& model = sim.model();
    model.linearizer().setContextOptions(GBFV_MODEL_IMMISCIBLE_2P, prm);
    model.newtonMethod().setTolerance(prm.newton_tolerance);
    model.newtonMethod().setIterationLimits(prm.newton_target_iterations, prm.newton_max_iterations);
    // initial solution from the problem's initial() (FvBaseDiscretization::applyInitialSolution)
    const int N = sim.gridView().size(0);
    model.solution(0).assign(N, LensGbfv::PrimaryVariables());
    Opm::ElementContext<LensGbfv> elemCtx(sim);
    for (const auto& e : Opm::elements(sim.gridView())) {
        elemCtx.updateStencil(e);
        sim.problem().initial(model.solution(0)[e.index], elemCtx, 0, 0);
    }
    model.solution(1) = model.solution(0);
    sim.setTimeStepSize(250.0);
    sim.beforeTimeStep = [&](Opm::Simulator<LensGbfv>& s) {
        if (s.timeStepIndex() == nanStep) s.model().solution(0)[N / 2][0] = std::nan("");
    };
    std::vector<double> stepDt;
    std::vector<int> stepNewton;
    int rc = 0;
    try {
        sim.run(steps, stepDt, stepNewton);
    }
    catch (const std::exception& ex) {
        std::fprintf(stderr, "run failed: %s\n", ex.what());
        rc = 1;
    }
    std::vector<double> x;
    for (const auto& pv : model.solution(0)) x.insert(x.end(), pv.begin(), pv.end());
    FILE* f = std::fopen(argv[4], "wb");
    if (!f) return 3;
    put(f, stepDt);
    put(f, stepNewton);
    put(f, x);
    put(f, std::vector<int64_t>{int64_t(sim.problem().failures), int64_t(model.linearizer().linearizations()),
                                int64_t(model.linearizer().residual().syncs()),
                                int64_t(model.linearizer().jacobian().syncs()),
                                int64_t(model.newtonMethod().hostSyncs()),
                                int64_t(model.newtonMethod().linearSolver().totalIterations())});
    std::fclose(f);
    return rc;
}
