// okl_equiv.cu -- the reference's device GatherScatter algorithm, restated in
// CUDA as a device-to-device baseline on the same GPU.  Not part of the
// library; bench.py times it beside the library's kernel.
//
// Algorithm of libs/ogs/okl/ogsKernels.okl:32-81 with the row blocks of
// ogsOperator.cpp:447-512 (blockSize 256, gatherNodesPerBlock 512,
// ogsOperator.hpp:122-123): rows are packed greedily, in row order, into
// blocks of at most 512 members; one 256-thread CTA per (block, component)
// stages the block's member values in shared memory, folds each row from the
// op identity over its members in ascending order, stages the row results,
// and writes every member back.  Sym GatherScatter uses the T maps for both
// sides (ogsOperator.cpp:327-332).  A row above 512 members is refused, as
// the reference aborts (ogsOperator.cpp:459-465).
//
// C ABI:  refdev_create(rowStarts[R+1], R, colIds) -> handle (NULL on error)
//         refdev_gather_scatter(h, d_q, K, type, op, stream) -> 0 or a CUDA error
//         refdev_nblocks(h), refdev_free(h)
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

namespace {

constexpr int kBlockSize = 256;
constexpr int kNodesPerBlock = 512;

// numeric_limits<T>::max() of the four field types
template <typename T> struct TypeMax;
template <> struct TypeMax<float> { __device__ static float get() { return 3.40282347e38f; } };
template <> struct TypeMax<double> { __device__ static double get() { return 1.7976931348623157e308; } };
template <> struct TypeMax<int32_t> { __device__ static int32_t get() { return 2147483647; } };
template <> struct TypeMax<long long> { __device__ static long long get() { return 9223372036854775807LL; } };

// op identities of ogsOperator.cpp:36-55: 0, 1, -max, +max
template <typename T, int OP>
__device__ __forceinline__ T identity() {
  if (OP == 0) return T(0);
  if (OP == 1) return T(1);
  if (OP == 2) return -TypeMax<T>::get();
  return TypeMax<T>::get();
}

template <typename T, int OP>
__device__ __forceinline__ void apply(T& a, const T b) {
  if (OP == 0) a += b;
  else if (OP == 1) a *= b;
  else if (OP == 2) { if (b > a) a = b; }
  else { if (b < a) a = b; }
}

template <typename T, int OP>
__global__ void __launch_bounds__(kBlockSize) okl_gather_scatter(const int32_t* __restrict__ blockStarts,
                                                                 const int32_t* __restrict__ starts,
                                                                 const int32_t* __restrict__ ids, int K, T* q) {
  __shared__ T gtemp[kNodesPerBlock];
  __shared__ T stemp[kNodesPerBlock];
  const int b = blockIdx.x;
  const int k = blockIdx.y;
  const int r0 = blockStarts[b], r1 = blockStarts[b + 1];
  const int e0 = starts[r0], e1 = starts[r1];
  for (int e = e0 + threadIdx.x; e < e1; e += kBlockSize) gtemp[e - e0] = q[k + static_cast<int64_t>(ids[e]) * K];
  __syncthreads();
  for (int r = r0 + threadIdx.x; r < r1; r += kBlockSize) {
    const int a0 = starts[r] - e0, a1 = starts[r + 1] - e0;
    T acc = identity<T, OP>();
    for (int e = a0; e < a1; ++e) apply<T, OP>(acc, gtemp[e]);
    for (int e = a0; e < a1; ++e) stemp[e] = acc;
  }
  __syncthreads();
  for (int e = e0 + threadIdx.x; e < e1; e += kBlockSize) q[k + static_cast<int64_t>(ids[e]) * K] = stemp[e - e0];
}

struct Handle {
  int nblocks = 0;
  int32_t* d_blocks = nullptr;
  int32_t* d_starts = nullptr;
  int32_t* d_ids = nullptr;
};

template <typename T>
cudaError_t launch_typed(const Handle* h, void* q, int K, int op, cudaStream_t s) {
  const dim3 grid(static_cast<unsigned>(h->nblocks), static_cast<unsigned>(K));
  T* v = static_cast<T*>(q);
  switch (op) {
    case 0: okl_gather_scatter<T, 0><<<grid, kBlockSize, 0, s>>>(h->d_blocks, h->d_starts, h->d_ids, K, v); break;
    case 1: okl_gather_scatter<T, 1><<<grid, kBlockSize, 0, s>>>(h->d_blocks, h->d_starts, h->d_ids, K, v); break;
    case 2: okl_gather_scatter<T, 2><<<grid, kBlockSize, 0, s>>>(h->d_blocks, h->d_starts, h->d_ids, K, v); break;
    default: okl_gather_scatter<T, 3><<<grid, kBlockSize, 0, s>>>(h->d_blocks, h->d_starts, h->d_ids, K, v); break;
  }
  return cudaGetLastError();
}

}  // namespace

extern "C" {

void* refdev_create(const int32_t* rowStarts, int64_t R, const int32_t* colIds) {
  if (R < 0 || (R > 0 && (!rowStarts || !colIds))) return nullptr;
  std::vector<int32_t> blocks;
  if (R > 0) blocks.push_back(0);
  int64_t sum = 0;
  for (int64_t r = 0; r < R; ++r) {
    const int64_t d = rowStarts[r + 1] - rowStarts[r];
    if (d > kNodesPerBlock) return nullptr;
    if (sum + d > kNodesPerBlock) {
      blocks.push_back(static_cast<int32_t>(r));
      sum = d;
    } else {
      sum += d;
    }
  }
  if (R > 0) blocks.push_back(static_cast<int32_t>(R));
  Handle* h = new Handle();
  h->nblocks = R > 0 ? static_cast<int>(blocks.size()) - 1 : 0;
  const int64_t nnz = R > 0 ? rowStarts[R] : 0;
  bool ok = cudaMalloc(&h->d_blocks, blocks.size() * 4 + 4) == cudaSuccess &&
            cudaMalloc(&h->d_starts, (R + 1) * 4) == cudaSuccess &&
            cudaMalloc(&h->d_ids, (nnz > 0 ? nnz : 1) * 4) == cudaSuccess;
  if (ok && R > 0)
    ok = cudaMemcpy(h->d_blocks, blocks.data(), blocks.size() * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(h->d_starts, rowStarts, (R + 1) * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
         (nnz == 0 || cudaMemcpy(h->d_ids, colIds, nnz * 4, cudaMemcpyHostToDevice) == cudaSuccess);
  if (!ok) {
    cudaFree(h->d_blocks);
    cudaFree(h->d_starts);
    cudaFree(h->d_ids);
    delete h;
    cudaGetLastError();
    return nullptr;
  }
  return h;
}

int refdev_nblocks(const void* hv) { return hv ? static_cast<const Handle*>(hv)->nblocks : 0; }

int refdev_gather_scatter(const void* hv, void* q, int K, int type, int op, void* stream) {
  const Handle* h = static_cast<const Handle*>(hv);
  if (!h || K < 1 || op < 0 || op > 3) return static_cast<int>(cudaErrorInvalidValue);
  if (h->nblocks == 0) return 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (type) {
    case 0: return static_cast<int>(launch_typed<float>(h, q, K, op, s));
    case 1: return static_cast<int>(launch_typed<double>(h, q, K, op, s));
    case 2: return static_cast<int>(launch_typed<int32_t>(h, q, K, op, s));
    case 3: return static_cast<int>(launch_typed<long long>(h, q, K, op, s));
    default: return static_cast<int>(cudaErrorInvalidValue);
  }
}

void refdev_free(void* hv) {
  Handle* h = static_cast<Handle*>(hv);
  if (!h) return;
  cudaFree(h->d_blocks);
  cudaFree(h->d_starts);
  cudaFree(h->d_ids);
  delete h;
}

}  // extern "C"
