// GMRES device loop (filled in by the GMRES implementation).
#include "solver.cuh"

namespace fsg {
int gmres_apply(Solver *s, Vec *, Vec *, fs_solve_info *) {
	return set_err(s->ctx, FS_ERR_UNSUPPORTED, "GMRES not built yet");
}
}  // namespace fsg
