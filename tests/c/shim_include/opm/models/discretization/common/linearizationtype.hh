// Test shim: the reference's linearization-type record
// (opm/models/discretization/common/linearizationtype.hh), restated with
// the same names so that include/gbfv_opm.hh compiles its TPFA interface
// against it.  Test infrastructure only.
#ifndef GBFV_TEST_SHIM_LINEARIZATIONTYPE_HH
#define GBFV_TEST_SHIM_LINEARIZATIONTYPE_HH

namespace Opm {

struct LinearizationType {
    enum VarType { implicit, pressure, seqtransport };
    VarType type = implicit;
    unsigned int time = 0;
};

}  // namespace Opm

#endif
