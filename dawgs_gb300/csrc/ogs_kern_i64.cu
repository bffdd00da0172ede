// ogs_kern_i64.cu -- int64_t instantiation of the tile kernels (one translation
// unit per value type so the four compile in parallel).
#include "ogs_kernels.cuh"

namespace ogsgb {
int launch_i64(const DevMaps& m, const FieldArgs& f, int mode, int op, Pattern pat, void* stream) {
  return launch_typed<int64_t>(m, f, mode, op, pat, stream);
}
}  // namespace ogsgb
