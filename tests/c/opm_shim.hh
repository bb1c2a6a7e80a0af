// Test shim of the reference types the adapter (include/gbfv_opm.hh) binds.
// The reference itself needs dune and opm-common, which are not installed,
// so this file restates, under the reference's names, exactly the parts the
// adapter touches:
//   - property lookup GetPropType<TypeTag, Properties::X> (here: the type
//     tag's member typedefs; the reference resolves the same names through
//     its property system, opm/models/utils/propertysystem.hh)
//   - a YaspGrid-like structured grid, its ECFV stencil and element /
//     boundary contexts (ecfvstencil.hh:150-415, fvbaseelementcontext.hh,
//     fvbaseboundarycontext.hh)
//   - NewtonMethod<TypeTag>: the apply() loop and default hooks of
//     opm/models/nonlinear/newtonmethod.hh:228-845, statement by statement
//     in the order that matters (timers and console output left out)
//   - the model's solution history, update / updateFailed / advanceTimeLevel
//     (fvbasediscretization.hh:1247-1400), FvBaseProblem::timeIntegration
//     (fvbaseproblem.hh:512-552) and the Simulator::run time loop
//     (simulator.hh:725-815)
//   - LensProblem's callbacks (tests/problems/lensproblem.hh:227-627)
// Test infrastructure only.
#ifndef GBFV_TEST_OPM_SHIM_HH
#define GBFV_TEST_OPM_SHIM_HH

#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

namespace Opm {

class NumericalProblem : public std::runtime_error {
public:
    using std::runtime_error::runtime_error;
};

namespace Properties {
struct Scalar {};
struct Simulator {};
struct Problem {};
struct Model {};
struct GridView {};
struct ElementContext {};
struct BoundaryContext {};
struct BoundaryRateVector {};
struct RateVector {};
struct Constraints {};
struct PrimaryVariables {};
struct SolutionVector {};
struct GlobalEqVector {};
struct Linearizer {};
struct LinearSolverBackend {};
struct NewtonMethod {};
}  // namespace Properties

template <class TypeTag, class Prop> struct PropOf;
#define GBFV_SHIM_PROP(P) \
    template <class T> struct PropOf<T, Properties::P> { using type = typename T::P; };
GBFV_SHIM_PROP(Scalar)
GBFV_SHIM_PROP(Simulator)
GBFV_SHIM_PROP(Problem)
GBFV_SHIM_PROP(Model)
GBFV_SHIM_PROP(GridView)
GBFV_SHIM_PROP(ElementContext)
GBFV_SHIM_PROP(BoundaryContext)
GBFV_SHIM_PROP(BoundaryRateVector)
GBFV_SHIM_PROP(RateVector)
GBFV_SHIM_PROP(Constraints)
GBFV_SHIM_PROP(PrimaryVariables)
GBFV_SHIM_PROP(SolutionVector)
GBFV_SHIM_PROP(GlobalEqVector)
GBFV_SHIM_PROP(Linearizer)
GBFV_SHIM_PROP(LinearSolverBackend)
GBFV_SHIM_PROP(NewtonMethod)
#undef GBFV_SHIM_PROP
template <class TypeTag, class Prop> using GetPropType = typename PropOf<TypeTag, Prop>::type;

// ------------------------------------------------------------ vectors -----
template <int n>
struct FieldVector : std::array<double, n> {
    FieldVector() { this->fill(0.0); }
    FieldVector(double v) { this->fill(v); }
    FieldVector& operator=(double v)
    {
        this->fill(v);
        return *this;
    }
    FieldVector& operator-=(const FieldVector& o)
    {
        for (int i = 0; i < n; ++i) (*this)[i] -= o[i];
        return *this;
    }
};
template <int n>
struct FieldMatrix {
    std::array<FieldVector<n>, n> r;
    FieldVector<n>& operator[](int i) { return r[i]; }
    const FieldVector<n>& operator[](int i) const { return r[i]; }
};

// Constraints of a DOF (FvBaseConstraints: primary variables + active flag)
template <int n>
struct Constraints : FieldVector<n> {
    bool active = false;
    bool isActive() const { return active; }
    void setActive(bool a) { active = a; }
};

// --------------------------------------------------------------- grid -----
// YaspGrid-like: cells i + nx*(j + ny*k), intersections -x,+x,-y,+y,-z,+z
template <int dim>
struct StructuredGridView {
    static constexpr int dimension = dim;
    static constexpr int dimensionworld = dim;
    std::array<int, 3> n{{1, 1, 1}};
    std::array<double, 3> len{{1.0, 1.0, 1.0}};
    int size(int codim) const { return codim == 0 ? n[0] * n[1] * n[2] : 0; }
    double h(int d) const { return len[d] / n[d]; }
    std::array<int, 3> coord(int I) const { return {{I % n[0], (I / n[0]) % n[1], I / (n[0] * n[1])}}; }
    int index(int i, int j, int k) const { return i + n[0] * (j + n[1] * k); }
};
struct Element {
    int index;
};
template <int dim>
struct ElementRange {
    int count;
    struct It {
        int i;
        Element operator*() const { return Element{i}; }
        It& operator++()
        {
            ++i;
            return *this;
        }
        bool operator!=(const It& o) const { return i != o.i; }
    };
    It begin() const { return It{0}; }
    It end() const { return It{count}; }
};
template <int dim>
ElementRange<dim> elements(const StructuredGridView<dim>& gv)
{
    return ElementRange<dim>{gv.size(0)};
}

// ECFV stencil of one element: DOF 0 = the element, then its neighbours
template <int dim>
class EcfvStencil {
public:
    using GlobalPosition = FieldVector<dim>;
    struct SubControlVolume {
        GlobalPosition pos;
        double vol = 0.0;
        const GlobalPosition& globalPos() const { return pos; }
        double volume() const { return vol; }
    };
    struct Face {
        unsigned short inIdx = 0, exIdx = 0;
        GlobalPosition ip, nrm;
        double a = 0.0;
        unsigned short interiorIndex() const { return inIdx; }
        unsigned short exteriorIndex() const { return exIdx; }
        const GlobalPosition& integrationPos() const { return ip; }
        const GlobalPosition& normal() const { return nrm; }
        double area() const { return a; }
    };
    void update(const StructuredGridView<dim>& gv, int I)
    {
        dofs_.assign(1, I);
        interior_.clear();
        boundary_.clear();
        const auto c = gv.coord(I);
        scv_.pos = GlobalPosition();
        scv_.vol = 1.0;
        for (int d = 0; d < dim; ++d) {
            scv_.pos[d] = (c[d] + 0.5) * gv.h(d);
            scv_.vol *= gv.h(d);
        }
        for (int d = 0; d < dim; ++d)
            for (int s = 0; s < 2; ++s) {
                Face f;
                f.nrm = GlobalPosition();
                f.nrm[d] = s ? 1.0 : -1.0;
                f.ip = scv_.pos;
                f.ip[d] += (s ? 0.5 : -0.5) * gv.h(d);
                f.a = scv_.vol / gv.h(d);
                const int cc = c[d] + (s ? 1 : -1);
                if (cc >= 0 && cc < gv.n[d]) {
                    auto nc = c;
                    nc[d] = cc;
                    f.exIdx = (unsigned short)dofs_.size();
                    dofs_.push_back(gv.index(nc[0], nc[1], nc[2]));
                    interior_.push_back(f);
                }
                else
                    boundary_.push_back(f);
            }
    }
    const SubControlVolume& subControlVolume(unsigned) const { return scv_; }
    size_t numInteriorFaces() const { return interior_.size(); }
    const Face& interiorFace(unsigned f) const { return interior_[f]; }
    size_t numBoundaryFaces() const { return boundary_.size(); }
    const Face& boundaryFace(unsigned f) const { return boundary_[f]; }
    size_t numDof() const { return dofs_.size(); }
    int globalSpaceIndex(unsigned dofIdx) const { return dofs_[dofIdx]; }

private:
    SubControlVolume scv_;
    std::vector<int> dofs_;
    std::vector<Face> interior_, boundary_;
};

template <class TypeTag>
class ElementContext {
    using Simulator = GetPropType<TypeTag, Properties::Simulator>;
    static constexpr int dim = GetPropType<TypeTag, Properties::GridView>::dimensionworld;

public:
    explicit ElementContext(const Simulator& sim) : sim_(sim) {}
    void updateStencil(const Element& e) { stencil_.update(sim_.gridView(), e.index); }
    const EcfvStencil<dim>& stencil(unsigned) const { return stencil_; }
    int globalSpaceIndex(unsigned dofIdx, unsigned) const { return stencil_.globalSpaceIndex(dofIdx); }
    const FieldVector<dim>& pos(unsigned dofIdx, unsigned) const
    {
        (void)dofIdx;
        return stencil_.subControlVolume(0).globalPos();
    }
    const Simulator& simulator() const { return sim_; }

private:
    const Simulator& sim_;
    EcfvStencil<dim> stencil_;
};

template <class TypeTag>
class BoundaryContext {
    using ElemCtx = GetPropType<TypeTag, Properties::ElementContext>;

public:
    explicit BoundaryContext(const ElemCtx& e) : elemCtx_(e) {}
    decltype(auto) pos(unsigned bfIdx, unsigned) const
    {
        return elemCtx_.stencil(0).boundaryFace(bfIdx).integrationPos();
    }
    const ElemCtx& elementContext() const { return elemCtx_; }

private:
    const ElemCtx& elemCtx_;
};

// ----------------------------------------------------------- Newton -------
// NewtonMethod<TypeTag> (newtonmethod.hh:157-845), the parts apply() runs.
template <class TypeTag>
class NewtonMethod {
    using Implementation = GetPropType<TypeTag, Properties::NewtonMethod>;
    using Simulator = GetPropType<TypeTag, Properties::Simulator>;
    using SolutionVector = GetPropType<TypeTag, Properties::SolutionVector>;
    using GlobalEqVector = GetPropType<TypeTag, Properties::GlobalEqVector>;
    using LinearSolverBackend = GetPropType<TypeTag, Properties::LinearSolverBackend>;

public:
    explicit NewtonMethod(Simulator& sim) : simulator_(sim), linearSolver_(sim) {}

    auto& model() { return simulator_.model(); }
    const auto& model() const { return simulator_.model(); }
    auto& problem() { return simulator_.problem(); }
    bool converged() const { return error_ <= tolerance(); }
    double tolerance() const { return tolerance_; }
    void setTolerance(double t) { tolerance_ = t; }
    int numIterations() const { return numIterations_; }
    LinearSolverBackend& linearSolver() { return linearSolver_; }

    // apply (newtonmethod.hh:228-438)
    bool apply()
    {
        SolutionVector& nextSolution = model().solution(/*historyIdx=*/0);
        SolutionVector currentSolution(nextSolution);
        GlobalEqVector solutionUpdate(nextSolution.size());
        auto& linearizer = model().linearizer();
        asImp_().begin_(nextSolution);
        try {
            while (asImp_().proceed_()) {
                asImp_().beginIteration_();
                currentSolution = nextSolution;
                asImp_().linearizeDomain_();
                asImp_().linearizeAuxiliaryEquations_();
                auto& residual = linearizer.residual();
                const auto& jacobian = linearizer.jacobian();
                linearSolver_.prepare(jacobian, residual);
                linearSolver_.setResidual(residual);
                linearSolver_.getResidual(residual);
                asImp_().preSolve_(currentSolution, residual);
                if (!asImp_().proceed_()) {
                    asImp_().endIteration_(nextSolution, currentSolution);
                    break;
                }
                linearSolver_.setMatrix(jacobian);
                solutionUpdate = GlobalEqVector(nextSolution.size());
                const bool converged = linearSolver_.solve(solutionUpdate);
                if (!converged) {
                    asImp_().failed_();
                    return false;
                }
                asImp_().postSolve_(currentSolution, residual, solutionUpdate);
                asImp_().update_(nextSolution, currentSolution, solutionUpdate, residual);
                asImp_().endIteration_(nextSolution, currentSolution);
            }
        }
        catch (const NumericalProblem&) {
            asImp_().failed_();
            return false;
        }
        asImp_().end_();
        if (!asImp_().converged()) {
            asImp_().failed_();
            return false;
        }
        asImp_().succeeded_();
        return true;
    }

    // suggestTimeStepSize (newtonmethod.hh:448-465)
    double suggestTimeStepSize(double oldDt) const
    {
        if (numIterations_ > targetIterations_) {
            const double percent = double(numIterations_ - targetIterations_) / targetIterations_;
            return std::max(problemMinTimeStep_, oldDt / (1.0 + percent));
        }
        const double percent = double(targetIterations_ - numIterations_) / targetIterations_;
        return std::max(problemMinTimeStep_, oldDt * (1.0 + percent / 1.2));
    }
    void setIterationLimits(int target, int max)
    {
        targetIterations_ = target;
        maxIterations_ = max;
    }

protected:
    void begin_(const SolutionVector&) { numIterations_ = 0; }
    void beginIteration_() { lastError_ = error_; }
    void linearizeDomain_() { model().linearizer().linearizeDomain(); }
    void linearizeAuxiliaryEquations_()
    {
        model().linearizer().linearizeAuxiliaryEquations();
        model().linearizer().finalize();
    }
    // the host versions of preSolve_ / postSolve_ / update_ are replaced by
    // the adapter; the shim keeps their signatures only
    template <class R>
    void preSolve_(const SolutionVector&, const R&)
    {
        throw std::logic_error("host preSolve_ is not used by the offload");
    }
    template <class R, class U>
    void postSolve_(const SolutionVector&, const R&, U&)
    {
    }
    template <class U, class R>
    void update_(SolutionVector&, const SolutionVector&, const U&, const R&)
    {
        throw std::logic_error("host update_ is not used by the offload");
    }
    void endIteration_(const SolutionVector&, const SolutionVector&) { ++numIterations_; }
    // proceed_ (newtonmethod.hh:788-806)
    bool proceed_() const
    {
        if (asImp_().numIterations() < 1) return true;
        if (asImp_().converged()) return false;
        if (asImp_().numIterations() >= maxIterations_) return error_ * 4.0 < lastError_;
        return true;
    }
    void end_() {}
    // failed_ (newtonmethod.hh:822-823)
    void failed_() { numIterations_ = targetIterations_ * 2; }
    void succeeded_() {}

    Implementation& asImp_() { return *static_cast<Implementation*>(this); }
    const Implementation& asImp_() const { return *static_cast<const Implementation*>(this); }

    Simulator& simulator_;
    LinearSolverBackend linearSolver_;
    double error_ = 0.0, lastError_ = 0.0, tolerance_ = 1e-8;
    int numIterations_ = 0;
    int targetIterations_ = 10, maxIterations_ = 20;
    double problemMinTimeStep_ = 0.0;
};

// ------------------------------------------------------------ model -------
template <class TypeTag>
class Model {
    using Simulator = GetPropType<TypeTag, Properties::Simulator>;
    using SolutionVector = GetPropType<TypeTag, Properties::SolutionVector>;
    using Linearizer = GetPropType<TypeTag, Properties::Linearizer>;
    using Newton = GetPropType<TypeTag, Properties::NewtonMethod>;

public:
    explicit Model(Simulator& sim) : newton_(sim) { linearizer_.init(sim); }
    SolutionVector& solution(unsigned t) { return sol_[t]; }
    const SolutionVector& solution(unsigned t) const { return sol_[t]; }
    Linearizer& linearizer() { return linearizer_; }
    const Linearizer& linearizer() const { return linearizer_; }
    Newton& newtonMethod() { return newton_; }
    const Newton& newtonMethod() const { return newton_; }
    size_t numGridDof() const { return sol_[0].size(); }
    // FvBaseDiscretization::update (fvbasediscretization.hh:1247-1320):
    // apply(), then updateFailed() when it did not converge
    bool update()
    {
        const bool converged = newton_.apply();
        if (!converged) updateFailed();
        return converged;
    }
    // updateFailed (:1362-1367)
    void updateFailed() { sol_[0] = sol_[1]; }
    // advanceTimeLevel (:1388-1400)
    void advanceTimeLevel() { sol_[1] = sol_[0]; }

private:
    Linearizer linearizer_;
    Newton newton_;
    SolutionVector sol_[2];
};

// --------------------------------------------------------- simulator ------
template <class TypeTag>
class Simulator {
    using Problem = GetPropType<TypeTag, Properties::Problem>;
    using ModelT = GetPropType<TypeTag, Properties::Model>;
    using GridViewT = GetPropType<TypeTag, Properties::GridView>;

public:
    explicit Simulator(const GridViewT& gv) : gridView_(gv), problem_(*this), model_(*this) {}
    const GridViewT& gridView() const { return gridView_; }
    Problem& problem() { return problem_; }
    const Problem& problem() const { return problem_; }
    ModelT& model() { return model_; }
    const ModelT& model() const { return model_; }
    double timeStepSize() const { return dt_; }
    void setTimeStepSize(double dt) { dt_ = dt; }
    double time() const { return time_; }
    int timeStepIndex() const { return step_; }
    // called before every time step (the test's fault injection point)
    std::function<void(Simulator&)> beforeTimeStep;

    // the time loop of Simulator::run (simulator.hh:725-815): integrate,
    // advance the time level, take the next dt from the Newton method
    void run(int steps, std::vector<double>& stepDt, std::vector<int>& stepNewton)
    {
        for (int s = 0; s < steps; ++s) {
            if (beforeTimeStep) beforeTimeStep(*this);
            problem_.timeIntegration();
            stepDt.push_back(dt_);
            stepNewton.push_back(model_.newtonMethod().numIterations());
            const double oldDt = dt_;
            model_.advanceTimeLevel();
            time_ += oldDt;
            ++step_;
            dt_ = problem_.nextTimeStepSize();
        }
    }

private:
    GridViewT gridView_;
    Problem problem_;
    ModelT model_;
    double dt_ = 0.0, time_ = 0.0;
    int step_ = 0;
};

}  // namespace Opm

#endif  // GBFV_TEST_OPM_SHIM_HH
