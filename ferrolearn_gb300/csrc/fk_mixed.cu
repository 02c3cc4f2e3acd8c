// fk_mixed.cu -- mixed-precision assignment (approximate pass + exact FP64
// re-check). Placeholder until the approximate kernels land.
#include "fk_internal.cuh"

namespace fk {

template <typename TX>
void run_assign_mixed(Ctx &, const TX *, int64_t, int, const double *, int, int, int32_t *, double *, DevScalars *,
                      bool) {
    set_error("mixed precision is not built yet");
    fail(FK_ERR_UNSUPPORTED);
}

template <typename TX>
void launch_mixed_inertia(Ctx &, const SortPlan &, const TX *, int, const int32_t *, const int32_t *, const double *,
                          DevScalars *) {
    set_error("mixed precision is not built yet");
    fail(FK_ERR_UNSUPPORTED);
}

template void run_assign_mixed<float>(Ctx &, const float *, int64_t, int, const double *, int, int, int32_t *,
                                      double *, DevScalars *, bool);
template void run_assign_mixed<double>(Ctx &, const double *, int64_t, int, const double *, int, int, int32_t *,
                                       double *, DevScalars *, bool);
template void launch_mixed_inertia<float>(Ctx &, const SortPlan &, const float *, int, const int32_t *,
                                          const int32_t *, const double *, DevScalars *);
template void launch_mixed_inertia<double>(Ctx &, const SortPlan &, const double *, int, const int32_t *,
                                           const int32_t *, const double *, DevScalars *);

}  // namespace fk
