// Family construction on the GPU: the member search of pdsolve::setDatModel
// (the block-hashed neighbour search, pdsolve.cpp:1442-1701), restated on the
// host in setup.cpp (build_setup).  A node j joins the family of node k when
// it lies in one of the 27 blocks around k's block, is not k itself, and is
// within k's horizon or k is within j's (the union rule); members keep the
// order of the host loop (blocks x-major, then y, then z; nodes in block
// insertion order), so the lists are identical to the host's.
//
// One warp per family.  Each pass over a block's node list tests 32 nodes at
// once and keeps the hits in order with a ballot and a prefix popcount; a
// count pass gives the offsets, a fill pass writes the members.  Distances
// use the host's operation order with explicit round-to-nearest products and
// sums (no fused multiply-add), so every borderline decision is the host's.
#include <cstdint>
#include <vector>

#include "model.h"
#include <cuda_runtime.h>

namespace pdx {

namespace {

struct FamArgs {
  const double* X;            // n_node x 3
  const double* delta_node;   // horizon of every node
  const int* fam_node;
  const double* fam_delta;
  const int* bptr;            // block b holds bnodes[bptr[b] .. bptr[b+1])
  const int* bnodes;
  double lbc[3];
  double block_size;
  int nb[3];
  double eps;                 // md * md * 1e-16
  int nf;
  const int64_t* off;         // fill pass: offsets of each family
  int* members;               // fill pass: output
  int* count;                 // count pass: members of each family (with k)
};

__device__ __forceinline__ double sq(double a) { return __dmul_rn(a, a); }

template <bool kFill>
__global__ void __launch_bounds__(256) k_family(FamArgs a) {
  const int f = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (f >= a.nf) return;   // whole warps leave together (nf is per warp)
  const int k = a.fam_node[f];
  const double xk0 = a.X[(size_t)k * 3], xk1 = a.X[(size_t)k * 3 + 1], xk2 = a.X[(size_t)k * 3 + 2];
  const double dk = a.fam_delta[f];
  const double dk2 = __dadd_rn(sq(dk), a.eps);
  int ib[3];
  ib[0] = (int)__ddiv_rn(__dsub_rn(xk0, a.lbc[0]), a.block_size);
  ib[1] = (int)__ddiv_rn(__dsub_rn(xk1, a.lbc[1]), a.block_size);
  ib[2] = (int)__ddiv_rn(__dsub_rn(xk2, a.lbc[2]), a.block_size);
  int64_t pos = kFill ? a.off[f] : 0;
  if (kFill && lane == 0) a.members[pos] = k;
  pos += 1;
  const unsigned below = (1u << lane) - 1u;
  for (int x = ib[0] - 1; x < ib[0] + 2; x++)
    for (int y = ib[1] - 1; y < ib[1] + 2; y++)
      for (int z = ib[2] - 1; z < ib[2] + 2; z++) {
        if (x < 0 || x >= a.nb[0] || y < 0 || y >= a.nb[1] || z < 0 || z >= a.nb[2]) continue;
        const int b = x + y * a.nb[0] + z * a.nb[0] * a.nb[1];
        const int i1 = a.bptr[b + 1];
        for (int i0 = a.bptr[b]; i0 < i1; i0 += 32) {
          const int i = i0 + lane;
          bool hit = false;
          int j = -1;
          if (i < i1) {
            j = a.bnodes[i];
            const double* xm = a.X + (size_t)j * 3;
            const double dist =
                __dadd_rn(__dadd_rn(sq(__dsub_rn(xm[0], xk0)), sq(__dsub_rn(xm[1], xk1))), sq(__dsub_rn(xm[2], xk2)));
            const double dj2 = __dadd_rn(sq(a.delta_node[j]), a.eps);
            hit = dist > a.eps && (dist < dk2 || dist < dj2);
          }
          const unsigned mask = __ballot_sync(0xffffffffu, hit);
          if (kFill && hit) a.members[pos + __popc(mask & below)] = j;
          pos += __popc(mask);
        }
      }
  if (!kFill && lane == 0) a.count[f] = (int)pos;
}

struct DevArrays {
  std::vector<void*> ptrs;
  template <typename T>
  T* put(const T* src, size_t n, cudaStream_t s) {
    void* p = nullptr;
    if (cudaMalloc(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    if (n) cudaMemcpyAsync(p, src, n * sizeof(T), cudaMemcpyHostToDevice, s);
    return static_cast<T*>(p);
  }
  ~DevArrays() {
    for (void* p : ptrs) cudaFree(p);
  }
};

}  // namespace

bool gpu_family_search(const Mesh& m, Setup& s, const std::vector<double>& delta_node, double md, int device,
                       Error& err) {
  auto fail = [&](const char* what, cudaError_t e) {
    err.code = 7;
    err.msg = std::string("family search on the GPU: ") + what + ": " + cudaGetErrorString(e);
    return false;
  };
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail("device", e);
  const int nf = (int)s.fam_node.size();
  const size_t nblk = s.block_nodes.size();
  std::vector<int> bptr(nblk + 1, 0), bnodes;
  bnodes.reserve((size_t)m.n_node);
  for (size_t b = 0; b < nblk; b++) {
    bnodes.insert(bnodes.end(), s.block_nodes[b].begin(), s.block_nodes[b].end());
    bptr[b + 1] = (int)bnodes.size();
  }
  cudaStream_t st;
  if ((e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess) return fail("stream", e);
  bool ok = false;
  {
    DevArrays d;
    FamArgs a{};
    a.X = d.put(m.X.data(), m.X.size(), st);
    a.delta_node = d.put(delta_node.data(), delta_node.size(), st);
    a.fam_node = d.put(s.fam_node.data(), s.fam_node.size(), st);
    a.fam_delta = d.put(s.fam_delta.data(), s.fam_delta.size(), st);
    a.bptr = d.put(bptr.data(), bptr.size(), st);
    a.bnodes = d.put(bnodes.data(), bnodes.size(), st);
    std::vector<int> count(nf);
    a.count = d.put(count.data(), count.size(), st);
    for (int i = 0; i < 3; i++) {
      a.lbc[i] = s.lbc[i];
      a.nb[i] = s.nblocks[i];
    }
    a.block_size = s.block_size;
    a.eps = md * md * 1.0e-16;
    a.nf = nf;
    if (!a.X || !a.delta_node || !a.fam_node || !a.fam_delta || !a.bptr || !a.bnodes || !a.count) {
      cudaStreamDestroy(st);
      return fail("allocation", cudaErrorMemoryAllocation);
    }
    const int threads = 256;
    const int grid = (int)(((int64_t)nf * 32 + threads - 1) / threads);
    if (nf) k_family<false><<<grid, threads, 0, st>>>(a);
    if (nf) cudaMemcpyAsync(count.data(), a.count, (size_t)nf * sizeof(int), cudaMemcpyDeviceToHost, st);
    e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) {
      s.fam_off.assign((size_t)nf + 1, 0);
      for (int f = 0; f < nf; f++) s.fam_off[(size_t)f + 1] = s.fam_off[f] + count[f];
      s.fam_members.assign((size_t)s.fam_off[nf], 0);
      a.off = d.put(s.fam_off.data(), s.fam_off.size(), st);
      int* dm = nullptr;
      if (a.off && cudaMalloc(&dm, (s.fam_members.size() ? s.fam_members.size() : 1) * sizeof(int)) == cudaSuccess) {
        d.ptrs.push_back(dm);
        a.members = dm;
        if (nf) k_family<true><<<grid, threads, 0, st>>>(a);
        if (!s.fam_members.empty())
          cudaMemcpyAsync(s.fam_members.data(), dm, s.fam_members.size() * sizeof(int), cudaMemcpyDeviceToHost, st);
        e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) e = cudaGetLastError();
        ok = e == cudaSuccess;
      } else {
        e = cudaErrorMemoryAllocation;
      }
    }
  }
  cudaStreamDestroy(st);
  if (!ok) return fail("kernel", e);
  return true;
}

}  // namespace pdx
