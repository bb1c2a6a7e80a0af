/*
 * gbfv_opm.hh -- the reference-side adapter: three classes that implement the
 * interfaces OPM/opm-models selects through its property system, over one
 * gbfv_ctx* of the C ABI (gbfv.h).  Header-only C++17; compiled with the
 * reference's headers (the including file provides Opm::GetPropType,
 * Opm::Properties::*, Opm::NewtonMethod and Opm::NumericalProblem) and linked
 * with -lgbfv.
 *
 * What each class replaces (paths inside OPM/opm-models):
 *   GbfvLinearizer<TypeTag>  Properties::Linearizer: FvBaseLinearizer
 *                            (opm/models/discretization/common/
 *                            fvbaselinearizer.hh:133-375)
 *   GbfvBackend<TypeTag>     Properties::LinearSolverBackend: the backend
 *                            interface of ParallelBaseBackend
 *                            (opm/simulators/linalg/parallelbasebackend.hh:
 *                            137-290)
 *   GbfvNewtonMethod<TypeTag, Parent>
 *                            Properties::NewtonMethod: keeps the reference's
 *                            NewtonMethod::apply loop (opm/models/nonlinear/
 *                            newtonmethod.hh:228-438) and overrides its hooks
 *   GbfvBoundaryRateVector<TypeTag>
 *                            Properties::BoundaryRateVector: records what the
 *                            problem's boundary() sets (setFreeFlow /
 *                            setMassRate / setNoFlow, immiscibleboundary-
 *                            ratevector.hh:97-213) so the description of the
 *                            boundary can be handed to the device
 *   gbfvContext<TypeTag>(simulator)
 *                            builds the gbfv_problem from the grid view, the
 *                            ECFV stencils (ecfvstencil.hh:389-415) and the
 *                            problem's callbacks: intrinsicPermeability,
 *                            porosity, materialLawParams, temperature,
 *                            boundary, constraints (lensproblem.hh:356-548)
 *
 * State: the device holds the authoritative primary variables during a time
 * step.  begin_ uploads model().solution(0) (after a failed attempt the
 * model's updateFailed has reset it to solution(1),
 * fvbasediscretization.hh:1362-1367, so the retry starts from the old time
 * level); end_ copies the converged state back into solution(0) before the
 * time loop's advanceTimeLevel (fvbasediscretization.hh:1388-1400) shifts it
 * into solution(1).  The device's old time level is the storage cached at
 * Newton iteration 0 from the state begin_ uploaded, so advanceTimeLevel
 * needs no device call.  Inside apply() the reference copies nextSolution
 * into currentSolution each iteration; those host copies are not read by the
 * offloaded hooks.
 *
 * Mirrors: residual() and jacobian() return views whose host copies are
 * filled only when the caller reads them (GbfvResidualView::host(),
 * GbfvJacobianView::istlBlocks()); apply() only passes them on to the
 * backend and the hooks, which work on the device, so no Jacobian crosses
 * to the host during a Newton iteration.
 *
 * Errors: numerical status codes (GBFV_ERR_NUMERICAL, _NONFINITE,
 * _BREAKDOWN, _NOT_CONVERGED, _SINGULAR) become Opm::NumericalProblem, which
 * apply() catches (newtonmethod.hh:381-395) so the time loop halves dt
 * (fvbaseproblem.hh:512-552); everything else is std::runtime_error.
 */
#ifndef GBFV_OPM_HH
#define GBFV_OPM_HH

#include "gbfv.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

// the reference's linearization-type record, used by the TPFA linearizer's
// interface (tpfalinearizer.hh:300-306)
#if __has_include(<opm/models/discretization/common/linearizationtype.hh>)
#include <opm/models/discretization/common/linearizationtype.hh>
#define GBFV_OPM_HAVE_LINEARIZATION_TYPE 1
#endif

namespace Opm {

// ------------------------------------------------------------ errors ------
inline void gbfvCheck(int st, const char* where)
{
    if (st == GBFV_OK) return;
    const std::string msg = std::string(where) + ": status " + std::to_string(st) + " " + gbfv_last_error();
    if (st == GBFV_ERR_NUMERICAL || st == GBFV_ERR_NONFINITE || st == GBFV_ERR_BREAKDOWN ||
        st == GBFV_ERR_NOT_CONVERGED || st == GBFV_ERR_SINGULAR)
        throw NumericalProblem(msg);
    throw std::runtime_error(msg);
}

// ---------------------------------------------------- boundary recorder ---
// Stands in for the model's BoundaryRateVector while the context is built:
// the problem's boundary() calls one of these setters per boundary face.
template <class TypeTag>
class GbfvBoundaryRateVector {
public:
    int kind = GBFV_BC_NOFLOW;
    std::array<double, 4> value{{0.0, 0.0, 0.0, 0.0}};
    bool haveFluids = false;
    double rho[2] = {0.0, 0.0}, mu[2] = {0.0, 0.0};

    // ImmiscibleBoundaryRateVector::setFreeFlow (immiscibleboundaryratevector.hh:97-160):
    // the boundary's fluid state; the device keeps p_w and S_w and evaluates the
    // boundary flux from them as the reference does
    template <class Context, class FluidState>
    void setFreeFlow(const Context&, unsigned, unsigned, const FluidState& fs)
    {
        kind = GBFV_BC_FREEFLOW;
        value = {{double(fs.pressure(0)), double(fs.saturation(0)), 0.0, 0.0}};
        for (int ph = 0; ph < 2; ++ph) {
            rho[ph] = double(fs.density(ph));
            mu[ph] = double(fs.viscosity(ph));
        }
        haveFluids = true;
    }
    // setMassRate (:162-180): rate per equation [kg/(m^2 s)]
    template <class Rate>
    void setMassRate(const Rate& rate)
    {
        kind = GBFV_BC_MASSRATE;
        value = {{0.0, 0.0, 0.0, 0.0}};
        for (unsigned e = 0; e < rate.size() && e < 4; ++e) value[e] = double(rate[e]);
    }
    // setNoFlow (:205-213)
    void setNoFlow()
    {
        kind = GBFV_BC_NOFLOW;
        value = {{0.0, 0.0, 0.0, 0.0}};
    }
};

// --------------------------------------------------- material parameters --
// The material-law parameter record of gbfv.h (GBFV_MAT_STRIDE doubles) from
// an opm-common parameter object: EffToAbsLawParams<RegularizedVanGenuchten>
// (residualSaturation(phase), vgAlpha(), vgN()) or <RegularizedBrooksCorey>
// (residualSaturation(phase), pcEntry(), lambda()).
namespace gbfv_detail {
template <class P, class = void> struct HasVg : std::false_type {};
template <class P>
struct HasVg<P, std::void_t<decltype(std::declval<const P&>().vgAlpha())>> : std::true_type {};
template <class P, class = void> struct HasBc : std::false_type {};
template <class P>
struct HasBc<P, std::void_t<decltype(std::declval<const P&>().pcEntry())>> : std::true_type {};
template <class PV, class = void> struct HasGasMeaning : std::false_type {};
template <class PV>
struct HasGasMeaning<PV, std::void_t<decltype(std::declval<const PV&>().primaryVarsMeaningGas())>>
    : std::true_type {};
}  // namespace gbfv_detail

template <class MaterialLawParams>
void gbfvMaterialRecord(const MaterialLawParams& p, double* out)
{
    std::fill(out, out + GBFV_MAT_STRIDE, 0.0);
    if constexpr (gbfv_detail::HasVg<MaterialLawParams>::value) {
        out[0] = GBFV_LAW_REG_VAN_GENUCHTEN;
        out[1] = double(p.residualSaturation(0));
        out[2] = double(p.residualSaturation(1));
        out[3] = double(p.vgAlpha());
        out[4] = double(p.vgN());
    }
    else if constexpr (gbfv_detail::HasBc<MaterialLawParams>::value) {
        out[0] = GBFV_LAW_REG_BROOKS_COREY;
        out[1] = double(p.residualSaturation(0));
        out[2] = double(p.residualSaturation(1));
        out[3] = double(p.pcEntry());
        out[4] = double(p.lambda());
    }
    else
        throw std::runtime_error("gbfvMaterialRecord: material law without van Genuchten or Brooks-Corey parameters");
}

// black-oil gas meaning of a PrimaryVariables object (BlackOilPrimaryVariables::
// primaryVarsMeaningGas, blackoilprimaryvariables.hh:138-143); immiscible: none
template <class PV>
int gbfvGasMeaning(const PV& pv)
{
    if constexpr (gbfv_detail::HasGasMeaning<PV>::value)
        return static_cast<int>(pv.primaryVarsMeaningGas());
    else {
        (void)pv;
        return 0;
    }
}
template <class PV>
void gbfvSetGasMeaning(PV& pv, int m)
{
    if constexpr (gbfv_detail::HasGasMeaning<PV>::value)
        pv.setPrimaryVarsMeaningGas(static_cast<decltype(pv.primaryVarsMeaningGas())>(m));
    else {
        (void)pv;
        (void)m;
    }
}

// ------------------------------------------------------- the description --
// The arrays a gbfv_problem points into, kept alive beside the context.
struct GbfvDescription {
    std::vector<double> center, volume, porosity, perm, connNormal, connCenter, connArea, bfNormal, bfCenter,
        bfArea, bfValue, matParams, constraintPv;
    std::vector<int32_t> material, connPtr, connNbr, connDir, bfPtr, bfType, constraint, constraintMeaning;
    gbfv_problem prob{};
};

// local intersection index (YaspGrid order -x,+x,-y,+y,-z,+z) of a face normal
template <class Vec>
int gbfvFaceDir(const Vec& n, int dim)
{
    int axis = 0;
    double best = -1.0;
    for (int d = 0; d < dim; ++d)
        if (std::abs(double(n[d])) > best) {
            best = std::abs(double(n[d]));
            axis = d;
        }
    return 2 * axis + (double(n[axis]) > 0.0 ? 1 : 0);
}

// Walk the grid once (FvBaseLinearizer::createMatrix_ does the same walk for
// the sparsity pattern, fvbaselinearizer.hh:418-452) and collect geometry,
// rock, material and boundary data through the problem's callbacks.
template <class TypeTag>
std::unique_ptr<GbfvDescription> gbfvDescribe(const GetPropType<TypeTag, Properties::Simulator>& sim, int model)
{
    using ElementContext = GetPropType<TypeTag, Properties::ElementContext>;
    using BoundaryRateVector = GetPropType<TypeTag, Properties::BoundaryRateVector>;
    static_assert(std::is_same_v<BoundaryRateVector, GbfvBoundaryRateVector<TypeTag>>,
                  "the offload type tag records boundary conditions with GbfvBoundaryRateVector");
    using BoundaryContext = GetPropType<TypeTag, Properties::BoundaryContext>;
    using Constraints = GetPropType<TypeTag, Properties::Constraints>;
    const auto& gridView = sim.gridView();
    const auto& problem = sim.problem();
    constexpr int dimWorld = std::decay_t<decltype(gridView)>::dimensionworld;
    auto D = std::make_unique<GbfvDescription>();
    const int N = int(gridView.size(0));
    D->center.assign(3 * size_t(N), 0.0);
    D->volume.assign(N, 0.0);
    D->porosity.assign(N, 0.0);
    D->perm.assign(3 * size_t(N), 0.0);
    D->material.assign(N, 0);
    D->connPtr.assign(N + 1, 0);
    D->bfPtr.assign(N + 1, 0);
    D->constraint.assign(N, -1);
    std::vector<std::vector<double>> matSeen;
    struct Conn { int nbr, dir; double n[3], c[3], a; };
    struct Bf { int type; double n[3], c[3], a, v[4]; };
    std::vector<std::vector<Conn>> conns(N);
    std::vector<std::vector<Bf>> bfs(N);
    bool haveFluids = false;
    double rho[2] = {0.0, 0.0}, mu[2] = {0.0, 0.0};
    double temperature = 0.0;
    ElementContext elemCtx(sim);
    for (const auto& elem : elements(gridView)) {
        elemCtx.updateStencil(elem);
        const auto& stencil = elemCtx.stencil(/*timeIdx=*/0);
        const int I = int(elemCtx.globalSpaceIndex(/*dofIdx=*/0, /*timeIdx=*/0));
        const auto& scv = stencil.subControlVolume(0);
        for (int d = 0; d < dimWorld; ++d) D->center[3 * size_t(I) + d] = double(scv.globalPos()[d]);
        D->volume[I] = double(scv.volume());
        D->porosity[I] = double(problem.porosity(elemCtx, 0, 0));
        const auto& K = problem.intrinsicPermeability(elemCtx, 0, 0);
        for (int d = 0; d < dimWorld; ++d) D->perm[3 * size_t(I) + d] = double(K[d][d]);
        temperature = double(problem.temperature(elemCtx, 0, 0));
        // materials: one record per distinct parameter set
        std::vector<double> rec(GBFV_MAT_STRIDE);
        gbfvMaterialRecord(problem.materialLawParams(elemCtx, 0, 0), rec.data());
        auto it = std::find(matSeen.begin(), matSeen.end(), rec);
        if (it == matSeen.end()) {
            matSeen.push_back(rec);
            it = matSeen.end() - 1;
        }
        D->material[I] = int32_t(it - matSeen.begin());
        // interior intersections (ECFV: one face per neighbour, exterior DOF index > 0)
        for (unsigned f = 0; f < stencil.numInteriorFaces(); ++f) {
            const auto& face = stencil.interiorFace(f);
            Conn c{};
            c.nbr = int(elemCtx.globalSpaceIndex(face.exteriorIndex(), 0));
            c.dir = gbfvFaceDir(face.normal(), dimWorld);
            for (int d = 0; d < dimWorld; ++d) {
                c.n[d] = double(face.normal()[d]);
                c.c[d] = double(face.integrationPos()[d]);
            }
            c.a = double(face.area());
            conns[I].push_back(c);
        }
        // boundary intersections and the problem's boundary conditions on them
        if (stencil.numBoundaryFaces() > 0) {
            BoundaryContext boundaryCtx(elemCtx);
            for (unsigned bf = 0; bf < stencil.numBoundaryFaces(); ++bf) {
                const auto& face = stencil.boundaryFace(bf);
                BoundaryRateVector values;
                problem.boundary(values, boundaryCtx, bf, 0);
                Bf b{};
                b.type = values.kind;
                for (int d = 0; d < dimWorld; ++d) {
                    b.n[d] = double(face.normal()[d]);
                    b.c[d] = double(face.integrationPos()[d]);
                }
                b.a = double(face.area());
                for (int e = 0; e < 4; ++e) b.v[e] = values.value[e];
                if (values.haveFluids && !haveFluids) {
                    haveFluids = true;
                    std::copy(values.rho, values.rho + 2, rho);
                    std::copy(values.mu, values.mu + 2, mu);
                }
                bfs[I].push_back(b);
            }
        }
        // constraints (FvBaseConstraints; wells of the reservoir problem)
        Constraints cons;
        problem.constraints(cons, elemCtx, 0, 0);
        if (cons.isActive()) {
            D->constraint[I] = int32_t(D->constraintMeaning.size());
            for (unsigned e = 0; e < 3; ++e) D->constraintPv.push_back(e < cons.size() ? double(cons[e]) : 0.0);
            D->constraintMeaning.push_back(gbfvGasMeaning(cons));
        }
    }
    for (int I = 0; I < N; ++I) {
        D->connPtr[I + 1] = D->connPtr[I] + int32_t(conns[I].size());
        D->bfPtr[I + 1] = D->bfPtr[I] + int32_t(bfs[I].size());
        for (const Conn& c : conns[I]) {
            D->connNbr.push_back(c.nbr);
            D->connDir.push_back(c.dir);
            D->connNormal.insert(D->connNormal.end(), c.n, c.n + 3);
            D->connCenter.insert(D->connCenter.end(), c.c, c.c + 3);
            D->connArea.push_back(c.a);
        }
        for (const Bf& b : bfs[I]) {
            D->bfType.push_back(b.type);
            D->bfNormal.insert(D->bfNormal.end(), b.n, b.n + 3);
            D->bfCenter.insert(D->bfCenter.end(), b.c, b.c + 3);
            D->bfArea.push_back(b.a);
            D->bfValue.insert(D->bfValue.end(), b.v, b.v + 4);
        }
    }
    for (const auto& m : matSeen) D->matParams.insert(D->matParams.end(), m.begin(), m.end());
    gbfv_problem& P = D->prob;
    std::memset(&P, 0, sizeof(P));
    P.model = model;
    P.num_cells = N;
    P.num_conn = int32_t(D->connNbr.size());
    P.num_bfaces = int32_t(D->bfType.size());
    P.center = D->center.data();
    P.volume = D->volume.data();
    P.porosity = D->porosity.data();
    P.perm = D->perm.data();
    P.material = D->material.data();
    P.conn_ptr = D->connPtr.data();
    P.conn_nbr = D->connNbr.data();
    P.conn_dir = D->connDir.data();
    P.conn_normal = D->connNormal.data();
    P.conn_center = D->connCenter.data();
    P.conn_area = D->connArea.data();
    P.bface_ptr = D->bfPtr.data();
    P.bface_normal = D->bfNormal.data();
    P.bface_center = D->bfCenter.data();
    P.bface_area = D->bfArea.data();
    P.bface_type = D->bfType.data();
    P.bface_value = D->bfValue.data();
    P.constraint = D->constraint.data();
    P.num_constraints = int32_t(D->constraintMeaning.size());
    P.constraint_pv = D->constraintPv.empty() ? nullptr : D->constraintPv.data();
    P.constraint_meaning = D->constraintMeaning.empty() ? nullptr : D->constraintMeaning.data();
    const auto& g = problem.gravity();
    for (int d = 0; d < dimWorld; ++d) P.gravity[d] = double(g[d]);
    P.num_materials = int32_t(matSeen.size());
    P.material_params = D->matParams.data();
    for (int ph = 0; ph < 2; ++ph) {
        P.rho[ph] = rho[ph];
        P.mu[ph] = mu[ph];
    }
    P.temperature = temperature;
    P.flux_module = GBFV_FLUX_DARCY;
    if (model == GBFV_MODEL_IMMISCIBLE_2P && !haveFluids)
        throw std::runtime_error("gbfvDescribe: no free-flow boundary gave the liquids' density and viscosity");
    return D;
}

// Run-time parameters the reference reads through Parameters::Get; the
// including translation unit may fill them from the reference's parameter
// system before the context is created.
inline gbfv_params gbfvDefaultParams()
{
    gbfv_params p;
    gbfv_default_params(&p);
    return p;
}

// ---------------------------------------------------------- linearizer ---
// residual(): the Newton residual; its host copy (natural order, [dof][eq])
// is filled on first read after each linearization.
class GbfvResidualView {
public:
    explicit GbfvResidualView(gbfv_ctx* ctx = nullptr) : ctx_(ctx) {}
    void bind(gbfv_ctx* ctx, size_t n, int b)
    {
        ctx_ = ctx;
        n_ = n;
        b_ = b;
        valid_ = false;
    }
    void invalidate() { valid_ = false; }
    size_t size() const { return n_; }
    const std::vector<double>& host() const
    {
        if (!valid_) {
            host_.resize(n_ * size_t(b_));
            gbfvCheck(gbfv_get_residual(ctx_, host_.data()), "gbfv_get_residual");
            valid_ = true;
            ++syncs_;
        }
        return host_;
    }
    double operator()(size_t dof, int eq) const { return host()[dof * size_t(b_) + eq]; }
    size_t syncs() const { return syncs_; }

private:
    gbfv_ctx* ctx_ = nullptr;
    size_t n_ = 0;
    int b_ = 0;
    mutable bool valid_ = false;
    mutable std::vector<double> host_;
    mutable size_t syncs_ = 0;
};

// jacobian(): the block-CSR Jacobian, copied to the host on first read
// after each linearization (istlBlocks: row_ptr, col_idx, row-major blocks,
// entry [eq][pv], as IstlSparseMatrixAdapter stores them)
class GbfvJacobianView {
public:
    void bind(gbfv_ctx* ctx, size_t n, int b, size_t nnz)
    {
        ctx_ = ctx;
        n_ = n;
        b_ = b;
        nnz_ = nnz;
        valid_ = false;
    }
    void invalidate() { valid_ = false; }
    size_t N() const { return n_; }
    size_t nonzeroes() const { return nnz_; }
    void istlBlocks(const int32_t** rowPtr, const int32_t** col, const double** blocks) const
    {
        if (!valid_) {
            rowPtr_.resize(n_ + 1);
            col_.resize(nnz_);
            blocks_.resize(nnz_ * size_t(b_) * size_t(b_));
            gbfvCheck(gbfv_get_jacobian(ctx_, rowPtr_.data(), col_.data(), blocks_.data()), "gbfv_get_jacobian");
            valid_ = true;
            ++syncs_;
        }
        *rowPtr = rowPtr_.data();
        *col = col_.data();
        *blocks = blocks_.data();
    }
    size_t syncs() const { return syncs_; }

private:
    gbfv_ctx* ctx_ = nullptr;
    size_t n_ = 0, nnz_ = 0;
    int b_ = 0;
    mutable bool valid_ = false;
    mutable std::vector<int32_t> rowPtr_, col_;
    mutable std::vector<double> blocks_;
    mutable size_t syncs_ = 0;
};

// FvBaseLinearizer's interface (fvbaselinearizer.hh:133-375).  Owns the
// context (one per simulator) and the description it was built from.
template <class TypeTag>
class GbfvLinearizer {
    using Simulator = GetPropType<TypeTag, Properties::Simulator>;

public:
    GbfvLinearizer() = default;
    GbfvLinearizer(const GbfvLinearizer&) = delete;
    GbfvLinearizer& operator=(const GbfvLinearizer&) = delete;
    ~GbfvLinearizer()
    {
        if (ctx_) gbfv_destroy(ctx_);
    }

    static void registerParameters() {}

    // init(simulator) (fvbaselinearizer.hh:147-160): the context is created on
    // first use, when the problem's parameters are in place
    void init(Simulator& sim) { sim_ = &sim; }

    // the model and run-time parameters of the context (before first use)
    void setContextOptions(int model, const gbfv_params& prm)
    {
        model_ = model;
        prm_ = prm;
    }

    gbfv_ctx* context()
    {
        if (!ctx_) {
            desc_ = gbfvDescribe<TypeTag>(*sim_, model_);
            int st = GBFV_OK;
            ctx_ = gbfv_create(&desc_->prob, &prm_, &st);
            if (!ctx_) gbfvCheck(st == GBFV_OK ? GBFV_ERR_CUDA : st, "gbfv_create");
            int n = 0, b = 0, nnz = 0;
            gbfvCheck(gbfv_dims(ctx_, &n, &b, &nnz), "gbfv_dims");
            residual_.bind(ctx_, size_t(n), b);
            jacobian_.bind(ctx_, size_t(n), b, size_t(nnz));
            numCells_ = n;
            blockSize_ = b;
        }
        return ctx_;
    }
    const GbfvDescription& description() const { return *desc_; }
    int numCells() const { return numCells_; }
    int blockSize() const { return blockSize_; }

    void eraseMatrix() {}
    void linearize()
    {
        linearizeDomain();
        linearizeAuxiliaryEquations();
        finalize();
    }
    // linearizeDomain (fvbaselinearizer.hh:201-241): the storage cache reads
    // the time step size and the Newton iteration (fvbaselocalresidual.hh:535-571)
    void linearizeDomain()
    {
        gbfv_ctx* c = context();
        gbfvCheck(gbfv_set_timestep(c, double(sim_->timeStepSize())), "gbfv_set_timestep");
        gbfvCheck(gbfv_set_newton_iteration(c, sim_->model().newtonMethod().numIterations()),
                  "gbfv_set_newton_iteration");
        gbfvCheck(gbfv_linearize(c), "gbfv_linearize");
        residual_.invalidate();
        jacobian_.invalidate();
        ++linearizations_;
    }
    void linearizeAuxiliaryEquations() {}
    void finalize() {}
    void updateDiscretizationParameters() {}
    void updateBoundaryConditionData() {}
    void updateFlowsInfo() {}

    GbfvResidualView& residual() { return residual_; }
    const GbfvResidualView& residual() const { return residual_; }
    const GbfvJacobianView& jacobian() const { return jacobian_; }
    size_t linearizations() const { return linearizations_; }

private:
    Simulator* sim_ = nullptr;
    gbfv_ctx* ctx_ = nullptr;
    std::unique_ptr<GbfvDescription> desc_;
    int model_ = GBFV_MODEL_IMMISCIBLE_2P;
    gbfv_params prm_ = gbfvDefaultParams();
    int numCells_ = 0, blockSize_ = 0;
    GbfvResidualView residual_;
    GbfvJacobianView jacobian_;
    size_t linearizations_ = 0;
};

// ---------------------------------------------------- TPFA linearizer ----
// The Linearizer property of a TPFA type tag: TpfaLinearizer
// (tpfalinearizer.hh:116-370) with BlackOilLocalResidualTPFA, on the device
// path with params.linearizer = GBFV_LINEARIZER_TPFA (black-oil, automatic
// differentiation, no constraint cells).  Beyond the element linearizer's
// surface it carries TpfaLinearizer's: the linearization type (the device
// linearizes the fully implicit system; a pressure or sequential-transport
// request is refused), the flows / flores / velocity records (empty: they
// are filled only for the FLOWS, FLORES and DISPERC output of the
// reference's simulator, which this path does not write) and an empty
// constraints map (TpfaLinearizer applies none).
template <class TypeTag>
class GbfvTpfaLinearizer : public GbfvLinearizer<TypeTag> {
    using Base = GbfvLinearizer<TypeTag>;

public:
    void setContextOptions(int model, gbfv_params prm)
    {
        if (model != GBFV_MODEL_BLACKOIL_3P)
            throw std::runtime_error("GbfvTpfaLinearizer: the TPFA linearizer is the black-oil model's");
        prm.linearizer = GBFV_LINEARIZER_TPFA;
        Base::setContextOptions(model, prm);
    }

#ifdef GBFV_OPM_HAVE_LINEARIZATION_TYPE
    void setLinearizationType(LinearizationType t)
    {
        if (t.type != LinearizationType::implicit)
            throw std::runtime_error("GbfvTpfaLinearizer: only the fully implicit system is linearized on the device");
        linearizationType_ = t;
    }
    const LinearizationType& getLinearizationType() const { return linearizationType_; }
#endif

    const std::vector<double>& getFlowsInfo() const { return noRecords_; }
    const std::vector<double>& getFloresInfo() const { return noRecords_; }
    const std::vector<double>& getVelocityInfo() const { return noRecords_; }
    template <class Constraints = int>
    std::vector<std::pair<unsigned, Constraints>> constraintsMap() const
    {
        return {};
    }

private:
#ifdef GBFV_OPM_HAVE_LINEARIZATION_TYPE
    LinearizationType linearizationType_{};
#endif
    std::vector<double> noRecords_;
};

// ----------------------------------------------------- solver backend ----
// The backend interface (parallelbasebackend.hh:137-290).  The system never
// leaves the device: prepare / setResidual / setMatrix only mark it, solve()
// runs BiCGStab + ILU(0) on the device and leaves the update there for the
// Newton method's update_ (x, the host update vector, is not written).
template <class TypeTag>
class GbfvBackend {
    using Simulator = GetPropType<TypeTag, Properties::Simulator>;

public:
    explicit GbfvBackend(const Simulator& sim) : sim_(sim) {}
    static void registerParameters() {}
    void eraseMatrix() {}
    template <class M, class V> void prepare(const M&, const V&) {}
    template <class V> void setResidual(const V&) {}
    template <class V> void getResidual(V&) const {}
    template <class M> void setMatrix(const M&) {}
    // solve (parallelbicgstabbackend.hh:131-166): false when BiCGStab did not
    // converge or broke down, as the reference's backend returns
    template <class V>
    bool solve(V&)
    {
        int it = 0;
        gbfv_ctx* c = const_cast<Simulator&>(sim_).model().linearizer().context();
        const int st = gbfv_solve(c, nullptr, &it);
        iterations_ = size_t(it);
        totalIterations_ += size_t(it);
        if (st == GBFV_ERR_NOT_CONVERGED || st == GBFV_ERR_BREAKDOWN) return false;
        gbfvCheck(st, "gbfv_solve");
        return true;
    }
    size_t iterations() const { return iterations_; }
    size_t totalIterations() const { return totalIterations_; }
    void resetTotalIterations() { totalIterations_ = 0; }

private:
    const Simulator& sim_;
    size_t iterations_ = 0, totalIterations_ = 0;
};

// ------------------------------------------------------ Newton method ----
// The reference's apply() loop with the device doing the error, the update
// (chop + primary-variable switching) and holding the state.  Parent is
// NewtonMethod<TypeTag> (immiscible) or BlackOilNewtonMethod<TypeTag>.
template <class TypeTag, class Parent>
class GbfvNewtonMethod : public Parent {
    using Simulator = GetPropType<TypeTag, Properties::Simulator>;
    // the apply() loop (NewtonMethod<TypeTag>) and a black-oil parent call the hooks
    friend Parent;
    friend class NewtonMethod<TypeTag>;

public:
    using Parent::Parent;

    // host copies of the device state made by end_ (for tests and logs)
    size_t hostSyncs() const { return hostSyncs_; }

protected:
    gbfv_ctx* ctx_() { return this->model().linearizer().context(); }

    // begin_ (newtonmethod.hh:514-521): the device takes model().solution(0)
    template <class SolutionVector>
    void begin_(const SolutionVector& u)
    {
        Parent::begin_(u);
        gbfv_ctx* c = ctx_();
        const int b = this->model().linearizer().blockSize();
        const size_t n = size_t(this->model().linearizer().numCells());
        pv_.resize(n * size_t(b));
        meaning_.resize(n);
        for (size_t i = 0; i < n; ++i) {
            for (int e = 0; e < b; ++e) pv_[i * size_t(b) + e] = double(u[i][e]);
            meaning_[i] = gbfvGasMeaning(u[i]);
        }
        gbfvCheck(gbfv_set_solution(c, pv_.data(), meaning_.data()), "gbfv_set_solution");
    }

    // preSolve_ (newtonmethod.hh:572-607): max |r * eqWeight| over the
    // unconstrained cells, on the device
    template <class SolutionVector, class Residual>
    void preSolve_(const SolutionVector&, const Residual&)
    {
        double err = 0.0;
        gbfvCheck(gbfv_newton_error(ctx_(), &err), "gbfv_newton_error");
        this->lastError_ = this->error_;
        this->error_ = err;
        if (this->error_ > maxError_)
            throw NumericalProblem("Newton: Error " + std::to_string(double(this->error_)) +
                                   " is larger than maximum allowed error of " + std::to_string(maxError_));
    }

    // postSolve_: the offloaded models have no auxiliary modules
    template <class SolutionVector, class Residual, class Update>
    void postSolve_(const SolutionVector&, const Residual&, Update&)
    {
    }

    // update_ (newtonmethod.hh:625-672) / BlackOilNewtonMethod::update_
    // (blackoilnewtonmethod.hh:176-199): x <- x - dx with chopping and
    // switching, on the device; the host nextSolution is written by end_
    template <class SolutionVector, class Update, class Residual>
    void update_(SolutionVector&, const SolutionVector&, const Update&, const Residual&)
    {
        int switched = 0;
        gbfvCheck(gbfv_newton_update(ctx_(), &switched), "gbfv_newton_update");
    }

    // end_ (newtonmethod.hh:808-812): the converged state back into solution(0)
    void end_()
    {
        Parent::end_();
        auto& u = this->model().solution(/*timeIdx=*/0);
        const int b = this->model().linearizer().blockSize();
        const size_t n = size_t(this->model().linearizer().numCells());
        pv_.resize(n * size_t(b));
        meaning_.resize(n);
        gbfvCheck(gbfv_get_solution(ctx_(), pv_.data(), meaning_.data()), "gbfv_get_solution");
        for (size_t i = 0; i < n; ++i) {
            for (int e = 0; e < b; ++e) u[i][e] = pv_[i * size_t(b) + e];
            gbfvSetGasMeaning(u[i], meaning_[i]);
        }
        ++hostSyncs_;
    }

public:
    // NewtonMaxError (newtonmethodparameters.hh); the reference reads it
    // through Parameters::Get in preSolve_
    void setMaxError(double e) { maxError_ = e; }

private:
    std::vector<double> pv_;
    std::vector<int32_t> meaning_;
    double maxError_ = 1e100;
    size_t hostSyncs_ = 0;
};

}  // namespace Opm

#endif  // GBFV_OPM_HH
