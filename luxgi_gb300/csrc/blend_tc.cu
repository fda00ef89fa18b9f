// Tensor-core (tcgen05) probe blend.  Placeholder until the kernel lands:
// the volume reports LUXGI_EUNSUPPORTED for the tensor blend.
#include "luxgi_internal.h"

namespace luxgi {

bool tc_blend_supported(const luxgi_ddgi_uniform&) { return false; }

cudaError_t launch_tc_blend(const TcBlendParams&, cudaStream_t) { return cudaErrorNotSupported; }

}  // namespace luxgi
