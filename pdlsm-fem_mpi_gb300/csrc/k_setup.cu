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
#include <climits>
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

// CSR pattern (build_csr_pattern in setup.cpp): node k interacts with the
// sorted, unique union of its family members and the nodes of its FE
// elements; each active DOF row of k holds the active DOFs of those nodes.
// One warp per node emits the union in increasing order by repeated warp
// minima over the candidates above the last one emitted (a node has at most
// a few hundred candidates), counting the row length in the count pass and
// writing the columns of all of k's rows in the fill pass.
struct PatArgs {
  int n_node, dim;
  const int* fam_of_node;
  const int64_t* fam_off;
  const int* fam_members;
  const int* ne_ptr;    // FE elements of node k: ne_list[ne_ptr[k] .. ne_ptr[k+1])
  const int* ne_list;
  const int* conn;      // 8 per element
  const int* elem_nn;
  const int* eq;        // n_node x dim, -1 for prescribed DOFs
  int64_t* rowlen;      // count pass: columns of each of node k's rows
  const int64_t* ia;    // fill pass
  int64_t* ja;
};

template <bool kFill>
__global__ void __launch_bounds__(256) k_pattern(PatArgs a) {
  const int k = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (k >= a.n_node) return;   // whole warps leave together
  const int D = a.dim;
  const int f = a.fam_of_node[k];
  const int64_t fb = f >= 0 ? a.fam_off[f] : 0;
  const int nfam = f >= 0 ? (int)(a.fam_off[f + 1] - fb) : 0;
  const int e0 = a.ne_ptr[k];
  const int total = nfam + (a.ne_ptr[k + 1] - e0) * 8;
  int64_t base = 0;   // fill pass: row start of lane's DOF (lanes < D)
  bool row = false;
  if (kFill && lane < D) {
    const int r = a.eq[(size_t)k * D + lane];
    row = r >= 0;
    if (row) base = a.ia[r];
  }
  int64_t p = 0;
  int last = -1;
  while (true) {
    int best = INT_MAX;
    for (int t = lane; t < total; t += 32) {
      int v;
      if (t < nfam) {
        v = a.fam_members[fb + t];
      } else {
        const int q = t - nfam;
        const int e = a.ne_list[e0 + (q >> 3)];
        v = (q & 7) < a.elem_nn[e] ? a.conn[(size_t)e * 8 + (q & 7)] : INT_MAX;
      }
      if (v > last && v < best) best = v;
    }
    best = __reduce_min_sync(0xffffffffu, best);
    if (best == INT_MAX) break;
    last = best;
    for (int jj = 0; jj < D; jj++) {
      const int c = a.eq[(size_t)best * D + jj];
      if (c < 0) continue;
      if (kFill && row) a.ja[base + p] = c;
      p++;
    }
  }
  if (!kFill && lane == 0) a.rowlen[k] = p;
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

bool gpu_csr_pattern(const Mesh& m, Setup& s, int device, Error& err) {
  auto fail = [&](const char* what, cudaError_t e) {
    err.code = 7;
    err.msg = std::string("CSR pattern on the GPU: ") + what + ": " + cudaGetErrorString(e);
    return false;
  };
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail("device", e);
  const int N = m.n_node, D = m.dim;
  // FE elements of every node
  std::vector<int> ne_ptr((size_t)N + 1, 0), ne_list;
  for (int el : s.fe)
    for (int j = 0; j < m.elem_nn[el]; j++) ne_ptr[(size_t)m.conn[(size_t)el * 8 + j] + 1]++;
  for (int k = 0; k < N; k++) ne_ptr[(size_t)k + 1] += ne_ptr[k];
  ne_list.resize((size_t)ne_ptr[N]);
  {
    std::vector<int> at(ne_ptr.begin(), ne_ptr.end() - 1);
    for (int el : s.fe)
      for (int j = 0; j < m.elem_nn[el]; j++) ne_list[(size_t)at[m.conn[(size_t)el * 8 + j]]++] = el;
  }
  cudaStream_t st;
  if ((e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess) return fail("stream", e);
  bool ok = false;
  {
    DevArrays d;
    PatArgs a{};
    a.n_node = N;
    a.dim = D;
    a.fam_of_node = d.put(s.fam_of_node.data(), s.fam_of_node.size(), st);
    a.fam_off = d.put(s.fam_off.data(), s.fam_off.size(), st);
    a.fam_members = d.put(s.fam_members.data(), s.fam_members.size(), st);
    a.ne_ptr = d.put(ne_ptr.data(), ne_ptr.size(), st);
    a.ne_list = d.put(ne_list.data(), ne_list.size(), st);
    a.conn = d.put(m.conn.data(), m.conn.size(), st);
    a.elem_nn = d.put(m.elem_nn.data(), m.elem_nn.size(), st);
    a.eq = d.put(s.eq.data(), s.eq.size(), st);
    std::vector<int64_t> rowlen((size_t)N);
    a.rowlen = d.put(rowlen.data(), rowlen.size(), st);
    if (!a.fam_of_node || !a.fam_off || !a.fam_members || !a.ne_ptr || !a.ne_list || !a.conn || !a.elem_nn || !a.eq ||
        !a.rowlen) {
      cudaStreamDestroy(st);
      return fail("allocation", cudaErrorMemoryAllocation);
    }
    const int threads = 256;
    const int grid = (int)(((int64_t)N * 32 + threads - 1) / threads);
    if (N) k_pattern<false><<<grid, threads, 0, st>>>(a);
    if (N) cudaMemcpyAsync(rowlen.data(), a.rowlen, (size_t)N * 8, cudaMemcpyDeviceToHost, st);
    e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) {
      // rows in equation order: node-major, DOF-minor
      s.csr_ia.assign((size_t)s.n_eq + 1, 0);
      for (int k = 0; k < N; k++)
        for (int i = 0; i < D; i++) {
          const int r = s.eq[(size_t)k * D + i];
          if (r >= 0) s.csr_ia[(size_t)r + 1] = rowlen[k];
        }
      for (int r = 0; r < s.n_eq; r++) s.csr_ia[(size_t)r + 1] += s.csr_ia[r];
      s.csr_ja.assign((size_t)s.csr_ia[s.n_eq], 0);
      a.ia = d.put(s.csr_ia.data(), s.csr_ia.size(), st);
      int64_t* dja = nullptr;
      if (a.ia && cudaMalloc(&dja, (s.csr_ja.size() ? s.csr_ja.size() : 1) * 8) == cudaSuccess) {
        d.ptrs.push_back(dja);
        a.ja = dja;
        if (N) k_pattern<true><<<grid, threads, 0, st>>>(a);
        if (!s.csr_ja.empty())
          cudaMemcpyAsync(s.csr_ja.data(), dja, s.csr_ja.size() * 8, cudaMemcpyDeviceToHost, st);
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
