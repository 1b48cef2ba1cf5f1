// Nodal (P1/P2) kernels and traction rows.
#include "common.cuh"

namespace mbem {

int nodal_matrix(int, const double*, int64_t, const double*, const double*, const double*, int64_t,
                 const double*, int order, double, int, double*, int64_t, void*) {
    return set_error(MBEM_ERR_UNSUPPORTED, "nodal matrices at order %d are not built", order);
}

int nodal_contract(int, const double*, int64_t, const double*, const double*, const double*, int64_t,
                   const double*, const double*, double, double, int order, double, int, double*, void*) {
    return set_error(MBEM_ERR_UNSUPPORTED, "nodal contractions at order %d are not built", order);
}

}  // namespace mbem

extern "C" int mbem_traction_matrix(const double*, const double*, int64_t, const double*, const double*,
                                    const double*, int64_t, const int64_t*, int64_t, double, double,
                                    int order, int, double, double*, int64_t, void*) {
    return mbem::set_error(MBEM_ERR_UNSUPPORTED, "traction rows at order %d are not built", order);
}
