// Consistency checks of a problem description (gbfv_problem) before a
// context reads it: offsets, counts, enum fields and table orderings.
//
// The reference gets the same data from objects that are consistent by
// construction (the Dune grid's element and intersection iterators,
// Problem::boundary/constraints/materialLawParams, the PVT tables that
// BlackOilFluidSystem::initFromState builds); through a C ABI they are plain
// arrays, so every offset the context follows is checked to stay inside the
// counts first.  Array lengths themselves are the caller's contract
// (include/gbfv.h states each one); what is checked is that the counts and
// offsets agree with one another.  Host code only, no device work: the
// checks run, and are tested, before a GPU is looked for.
#include <cmath>
#include <cstdint>
#include <string>

#include "../../include/gbfv.h"

namespace gbfv {
void setLastError(const std::string& s);

namespace {

int fail(const std::string& what)
{
    setLastError("problem description: " + what);
    return GBFV_ERR_ARG;
}

// ptr[0] == 0, non-decreasing, ptr[n] == total
bool offsetsOk(const int32_t* ptr, int n, int total)
{
    if (ptr[0] != 0 || ptr[n] != total) return false;
    for (int i = 0; i < n; ++i)
        if (ptr[i + 1] < ptr[i]) return false;
    return true;
}

// x[0] < x[1] < ... < x[n-1], all finite
bool increasing(const double* x, int n)
{
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(x[i]) || (i > 0 && !(x[i] > x[i - 1]))) return false;
    return true;
}

bool allPositive(const double* x, int n)
{
    for (int i = 0; i < n; ++i)
        if (!(x[i] > 0.0) || !std::isfinite(x[i])) return false;
    return true;
}

}  // namespace

int checkProblem(const gbfv_problem* P, int maxMaterials, int maxTable)
{
    if (!P) return fail("NULL");
    if (P->model != GBFV_MODEL_IMMISCIBLE_2P && P->model != GBFV_MODEL_BLACKOIL_3P) return fail("unknown model");
    const int N = P->num_cells;
    if (N <= 0) return fail("num_cells must be positive");
    if (N > GBFV_MAX_CELLS) {
        setLastError("grid larger than GBFV_MAX_CELLS (32-bit device indexing)");
        return GBFV_ERR_UNSUPPORTED;
    }
    if (P->num_elements < 0) return fail("negative num_elements");
    const bool vcfv = P->num_elements > 0;  // vertex-centred: the cells are the grid's vertices
    if (!P->center || !P->porosity || !P->perm || !P->material || !P->bface_ptr)
        return fail("incomplete (a required array is NULL)");
    if (!vcfv && (!P->volume || !P->conn_ptr || !P->conn_nbr || !P->conn_normal || !P->conn_center || !P->conn_area))
        return fail("incomplete (a required array is NULL)");
    if (P->flux_module != GBFV_FLUX_DARCY && P->flux_module != GBFV_FLUX_TRANS) return fail("unknown flux module");
    if (vcfv) {
        // elements: four corner vertices each; boundary faces grouped per
        // element, each on one of its element's corners
        if (P->num_conn != 0) return fail("a vertex-centred grid has no cell intersections (num_conn 0)");
        if (!P->elem_corner) return fail("elem_corner is NULL");
        for (int64_t k = 0; k < 4 * (int64_t)P->num_elements; ++k)
            if (P->elem_corner[k] < 0 || P->elem_corner[k] >= N)
                return fail("corner vertex out of range at element " + std::to_string(k / 4));
        if (P->num_bfaces < 0 || !offsetsOk(P->bface_ptr, P->num_elements, P->num_bfaces))
            return fail("bface_ptr must start at 0, not decrease and end at num_bfaces");
        if (P->num_bfaces > 0 && (!P->bface_corner || !P->bface_center || !P->bface_area))
            return fail("boundary faces need bface_corner, bface_center and bface_area");
        for (int f = 0; f < P->num_bfaces; ++f)
            if (P->bface_corner[f] < 0 || P->bface_corner[f] > 3)
                return fail("boundary face corner outside [0, 3] at face " + std::to_string(f));
        if (P->p1_gradients != 0 && P->p1_gradients != 1) return fail("p1_gradients must be 0 or 1");
    }
    else {
        // intersections: grouped per cell, the groups covering [0, count)
        if (P->num_conn < 0 || !offsetsOk(P->conn_ptr, N, P->num_conn))
            return fail("conn_ptr must start at 0, not decrease and end at num_conn");
        if (P->num_bfaces < 0 || !offsetsOk(P->bface_ptr, N, P->num_bfaces))
            return fail("bface_ptr must start at 0, not decrease and end at num_bfaces");
    }
    if (P->num_bfaces > 0 && !P->bface_normal) return fail("bface_normal is NULL");
    bool active = false;  // any boundary face other than no-flow
    if (P->bface_type)
        for (int f = 0; f < P->num_bfaces; ++f) {
            const int t = P->bface_type[f];
            if (t != GBFV_BC_NOFLOW && t != GBFV_BC_FREEFLOW && t != GBFV_BC_MASSRATE)
                return fail("unknown boundary type at face " + std::to_string(f));
            active |= t != GBFV_BC_NOFLOW;
        }
    if (active && (!P->bface_center || !P->bface_area || !P->bface_value))
        return fail("free-flow / mass-rate faces need bface_center, bface_area and bface_value");
    // materials: the law code an integer the context knows, every cell's index in range
    if (P->num_materials <= 0 || P->num_materials > maxMaterials)
        return fail("num_materials outside [1, " + std::to_string(maxMaterials) + "]");
    if (!P->material_params) return fail("material_params is NULL");
    for (int m = 0; m < P->num_materials; ++m) {
        const double law = P->material_params[(size_t)m * GBFV_MAT_STRIDE];
        // the immiscible model takes a two-phase law; the black-oil model's
        // relative permeabilities are Corey's, with the exponent of a
        // COREY3P record (2 for the two-phase records)
        const bool twoPhase = law == GBFV_LAW_REG_VAN_GENUCHTEN || law == GBFV_LAW_REG_BROOKS_COREY;
        if (!(twoPhase || (law == GBFV_LAW_COREY3P && P->model == GBFV_MODEL_BLACKOIL_3P)))
            return fail("material law of material " + std::to_string(m) + " unknown or not one of this model");
    }
    for (int i = 0; i < N; ++i)
        if (P->material[i] < 0 || P->material[i] >= P->num_materials)
            return fail("material index out of range at cell " + std::to_string(i));
    // constraints: -1 or a row of the constraint table
    if (P->num_constraints < 0) return fail("negative num_constraints");
    if (P->num_constraints > 0 && (!P->constraint_pv || !P->constraint_meaning))
        return fail("constraint_pv / constraint_meaning is NULL");
    if (P->constraint)
        for (int i = 0; i < N; ++i)
            if (P->constraint[i] < -1 || P->constraint[i] >= P->num_constraints)
                return fail("constraint row out of range at cell " + std::to_string(i));
    if (P->model == GBFV_MODEL_BLACKOIL_3P) {
        for (int k = 0; k < P->num_constraints; ++k) {
            const int g = P->constraint_meaning[k];
            if (g != GBFV_GAS_SG && g != GBFV_GAS_RS && g != GBFV_GAS_RV)
                return fail("unknown gas meaning of constraint " + std::to_string(k));
        }
        // PVT tables: sizes the device tables hold, pressures and R_s
        // increasing (R_s is also the abscissa of the bubble-point table),
        // formation volume factors positive (their inverses are tabulated)
        const gbfv_blackoil_pvt* t = P->pvt;
        if (!t) return fail("black-oil model without PVT tables");
        if (t->n_oil < 2 || t->n_oil > maxTable || t->n_gas < 2 || t->n_gas > maxTable)
            return fail("PVT table size outside [2, " + std::to_string(maxTable) + "]");
        if (!t->oil_p || !t->oil_rs || !t->oil_bo || !t->oil_mu || !t->gas_p || !t->gas_bg || !t->gas_mu)
            return fail("a PVT table column is NULL");
        if (!increasing(t->oil_p, t->n_oil) || !increasing(t->oil_rs, t->n_oil) || !increasing(t->gas_p, t->n_gas))
            return fail("PVT pressures and R_s must increase strictly");
        if (!allPositive(t->oil_bo, t->n_oil) || !allPositive(t->gas_bg, t->n_gas))
            return fail("PVT formation volume factors must be positive");
    }
    return GBFV_OK;
}

}  // namespace gbfv
