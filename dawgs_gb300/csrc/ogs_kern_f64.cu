// ogs_kern_f64.cu -- double instantiation of the tile kernels (one translation
// unit per value type so the four compile in parallel).
#include "ogs_kernels.cuh"

namespace ogsgb {
int launch_f64(const DevMaps& m, const FieldArgs& f, int mode, int op, Pattern pat, void* stream) {
  return launch_typed<double>(m, f, mode, op, pat, stream);
}
}  // namespace ogsgb
