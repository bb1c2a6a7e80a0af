// First of two C++ translation units that both include gbfv.h and link
// into one program with libgbfv.so: the header is valid C++ (its
// declarations carry C linkage) and defines nothing that would clash
// between units.
#include <cstring>

#include "gbfv.h"

// a problem description whose intersection offsets do not reach num_conn:
// gbfv_create must reject it before it looks for a device
int createInconsistentProblem()
{
    static const double center[3] = {0.5, 0.5, 0.0}, one[3] = {1.0, 1.0, 1.0};
    static const int32_t material[1] = {0}, connPtr[2] = {0, 0}, bfacePtr[2] = {0, 0};
    static const double matParams[GBFV_MAT_STRIDE] = {GBFV_LAW_REG_VAN_GENUCHTEN, 0.05, 0.0, 3.7e-3, 4.7};
    gbfv_problem p;
    std::memset(&p, 0, sizeof p);
    p.model = GBFV_MODEL_IMMISCIBLE_2P;
    p.num_cells = 1;
    p.num_conn = 3;  // conn_ptr ends at 0
    p.center = center;
    p.volume = one;
    p.porosity = one;
    p.perm = one;
    p.material = material;
    p.conn_ptr = connPtr;
    p.conn_nbr = material;
    p.conn_normal = one;
    p.conn_center = one;
    p.conn_area = one;
    p.bface_ptr = bfacePtr;
    p.num_materials = 1;
    p.material_params = matParams;
    int status = -1;
    gbfv_ctx* ctx = gbfv_create(&p, nullptr, &status);
    if (ctx) gbfv_destroy(ctx);
    return status;
}
