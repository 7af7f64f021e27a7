// Right preconditioners for the flexible GMRES cycle.
#include "krylov.hpp"

namespace cev {

size_t precond_workspace_size(const cev_fdfd_plan_s*, const cev_solve_opts&) { return 0; }

int precond_setup(Precond& pc, const cev_fdfd_plan_s*, const cev_solve_opts& o, const float*, int,
                  void*, cudaStream_t) {
  pc.kind = o.precond;
  CEV_REQUIRE(o.precond == CEV_PRECOND_NONE, "preconditioner %d is not available", o.precond);
  return CEV_OK;
}

int precond_apply(Precond&, const KCtx&, int, int, const float2*, float2*, cudaStream_t) {
  set_error("no preconditioner configured");
  return CEV_ERR_INVALID;
}

}  // namespace cev
