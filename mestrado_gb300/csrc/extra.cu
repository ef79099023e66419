// extra.cu -- release hook for the traceback / NJ state of a context.
#include "nwg_ctx.h"

namespace nwg {
void Ctx::extra_release() {}
}  // namespace nwg
