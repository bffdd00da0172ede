// ogs_kern_f64.cu -- double instantiation of the tile kernels (one translation
// unit per value type so the four compile in parallel).
#include "ogs_batch.cuh"
#include "ogs_launch.cuh"

namespace ogsgb {
int launch_f64(const DevMaps& m, const FieldArgs& f, int mode, int op, Pattern pat, void* stream) {
  return launch_typed<double>(m, f, mode, op, pat, stream);
}
int launch_batch_f64(const BatchEntry* E, const int64_t* starts, int n, int64_t nitems, int grid, int block,
                     int occ, int pipe, int plain, void* stream) {
  return launch_batch_typed<double>(E, starts, n, nitems, grid, block, occ, pipe, plain, stream);
}
int preload_batch_f64() { return preload_batch_shape<double, 256, 2>(); }

}  // namespace ogsgb
