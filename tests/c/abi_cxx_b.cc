// Second C++ translation unit (see abi_cxx_a.cc): the entry points that
// need no device, called from C++.
#include <cstdio>

#include "gbfv.h"

int createInconsistentProblem();

int main()
{
    gbfv_params p;
    gbfv_default_params(&p);
    if (p.precision != GBFV_PREC_FP64) return 1;
    if (gbfv_footprint_bytes(GBFV_MAX_CELLS + 1, 3, 3) != -1) return 2;
    if (createInconsistentProblem() != GBFV_ERR_ARG) return 3;
    std::printf("abi c++ ok: %s\n", gbfv_last_error());
    return 0;
}
