// Mixed-precision explicit step: forces in FP32, state, mass and update in
// FP64.  Same work split, failure order and update as the FP64 kernel
// (k_step.cu, k_step_common.cuh); the data it streams differ:
//
// Bond records (one per bond) are the only per-bond stream.  3D: 32 B = 6
// FP32 coefficients, the neighbour of the bond two places further in the
// lane's bond sequence (b + 2L: a family's lanes take bonds lane, lane + L,
// ...), and the bond's FP32 threshold, whose sign carries the bond state.
// Carrying the later bond's neighbour means a lane knows whom to gather
// next from a record that arrived an iteration ago, instead of waiting on
// the record it has just requested.  2D: 16 B = 3 coefficients + the bond's
// own neighbour, whose sign carries the state.  Records are prefetched two
// bonds ahead in registers.  Breaking a bond flips the sign in its record
// and clears the bit of the FP64 state array as well.
//
// Node records (2 float4 per node): [2n] = position (x, y, z, 0),
// [2n+1] = stored displacement (ux, uy, uz, varying-prescribed bits), so one
// 32-byte sector serves both the stretch test and the force.
//
// The stretch test runs in FP32 on the sqrt-free form (see k_step.cu); a bond
// within a relative band of 2e-4 around its threshold is settled after the
// bond loop by the reference's FP64 expression.
#include "k_step_common.cuh"

namespace pdx {

using namespace step;

namespace {

// 32-byte loads (one instruction per bond record or node record).  Bond
// records are read once per step: they bypass L1 and leave L2 first, so the
// node records the bonds gather stay cached.
struct Rec32 {
  float4 a, b;
};

__device__ __forceinline__ Rec32 ld_stream32(const float4* p) {
  Rec32 r;
  asm("ld.global.L1::no_allocate.L2::evict_first.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=f"(r.a.x), "=f"(r.a.y), "=f"(r.a.z), "=f"(r.a.w), "=f"(r.b.x), "=f"(r.b.y), "=f"(r.b.z),
                 "=f"(r.b.w)
               : "l"(p));
  return r;
}

__device__ __forceinline__ Rec32 ld_keep32(const float4* p) {
  Rec32 r;
  asm("ld.global.L2::evict_last.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=f"(r.a.x), "=f"(r.a.y), "=f"(r.a.z), "=f"(r.a.w), "=f"(r.b.x), "=f"(r.b.y), "=f"(r.b.z),
                 "=f"(r.b.w)
               : "l"(p));
  return r;
}

__device__ __forceinline__ float4 ld_stream16(const float4* p) {
  float4 r;
  asm("ld.global.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
               : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
               : "l"(p));
  return r;
}

// PD-boundary correction of a bond, P du, from its FP32 record (2D: one
// float4 = 2x2 block; 3D: 8 floats in one 32-byte load + the ninth entry).
template <int D>
__device__ __forceinline__ void corr_apply(const DevView& v, int64_t slot, const float* du, float* acc) {
  if (D == 2) {
    const float4 c = ld_stream16(reinterpret_cast<const float4*>(v.corr32) + slot);
    acc[0] += c.x * du[0] + c.y * du[1];
    acc[1] += c.z * du[0] + c.w * du[1];
  } else {
    const Rec32 c = ld_stream32(reinterpret_cast<const float4*>(v.corr32) + 2 * slot);
    const float c8 = v.corr32_last[slot];
    acc[0] += c.a.x * du[0] + c.a.y * du[1] + c.a.z * du[D - 1];
    acc[1] += c.a.w * du[0] + c.b.x * du[1] + c.b.y * du[D - 1];
    acc[D - 1] += c.b.z * du[0] + c.b.w * du[1] + c8 * du[D - 1];
  }
}

// record of bond b (3D: 2 float4, 2D: 1)
template <int D>
__device__ __forceinline__ void load_record(const float4* R, int64_t b, float4& ra, float4& rb) {
  if (D == 3) {
    const Rec32 r = ld_stream32(R + 2 * b);
    ra = r.a;
    rb = r.b;
  } else {
    ra = ld_stream16(R + b);
  }
}

// Marks bond b broken in its record: 3D negates the threshold (positive for
// every intact bond), 2D stores the complement of the neighbour index.
template <int D>
__device__ __forceinline__ void mark_broken(float4* R, int64_t b, int m, float thr) {
  if (D == 3) reinterpret_cast<float*>(R + 2 * b + 1)[3] = -thr;
  else reinterpret_cast<int*>(R + b)[3] = ~m;
}

template <int D>
__device__ __forceinline__ void bond_force(const float4& ra, const float4& rb, const float* du, float* acc) {
  if (D == 2) {
    acc[0] += ra.x * du[0] + ra.y * du[1];
    acc[1] += ra.y * du[0] + ra.z * du[1];
  } else {
    acc[0] += ra.x * du[0] + ra.y * du[1] + ra.z * du[2];
    acc[1] += ra.y * du[0] + ra.w * du[1] + rb.x * du[2];
    acc[D - 1] += ra.z * du[0] + rb.x * du[1] + rb.y * du[2];
  }
}

// One 3D bond: FP32 stretch test (bonds within 2e-4 of the threshold are
// left to the FP64 pass after the loop) and, if it stays intact, its force.
struct Bond3Ctx {
  float4 xk, qk;
  float uk[3];
  float acc[3];
  int b0, corr0, nbroken;
  bool brk, force, deferred;
};

__device__ __forceinline__ void bond3(const DevView& v, float4* R, int b, const Rec32& r, const Rec32& g,
                                      Bond3Ctx& c) {
  if (!(r.b.w > 0.f)) return;               // broken
  const float4 um = g.b;
  if (c.brk) {
    const float4 xm = g.a;
    const float x0 = xm.x - c.xk.x, x1 = xm.y - c.xk.y, x2 = xm.z - c.xk.z;
    const float e0 = um.x - c.qk.x, e1 = um.y - c.qk.y, e2 = um.z - c.qk.z;
    const float lhs = 2.f * (x0 * e0 + x1 * e1 + x2 * e2) + (e0 * e0 + e1 * e1 + e2 * e2);
    const float rhs = r.b.w;                // s0b (2 + s0b) |xi|^2
    if (fabsf(lhs - rhs) <= 2e-4f * rhs) {
      c.deferred = true;                    // settled in FP64 after the loop
      return;
    }
    if (lhs > rhs) {
      reinterpret_cast<float*>(R + 2 * (int64_t)b + 1)[3] = -rhs;
      atomicAnd(&v.state[b >> 5], ~(1u << (b & 31)));
      c.nbroken++;
      return;
    }
  }
  if (!c.force) return;
  float du[3] = {um.x, um.y, um.z};
  const unsigned fl = __float_as_uint(um.w);
  if (fl & 7u) {
    const int m = v.nbr[b];
#pragma unroll
    for (int i = 0; i < 3; i++)
      if ((fl >> i) & 1u) du[i] += (float)v.dtv[3 * m + i];
  }
#pragma unroll
  for (int i = 0; i < 3; i++) du[i] -= c.uk[i];
  bond_force<3>(r.a, r.b, du, c.acc);
  if (c.corr0 >= 0) corr_apply<3>(v, (int64_t)c.corr0 + (b - c.b0), du, c.acc);
}

// The 3D family loop of one lane: bonds b0 + lane, + L, ...  Unrolled by two
// with fixed register sets (A, B): while bond b is computed from set A, the
// record of b + L and the node record of its neighbour are in flight in set
// B.  The neighbour of b + L is known a bond earlier, from record b - L
// (records name the neighbour of the bond 2L further on), so the gather does
// not wait for the record it belongs to.
template <int L>
__device__ __forceinline__ void family_loop3(const DevView& v, float4* R, const float4* nr, int b, int b1,
                                             Bond3Ctx& c) {
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  Rec32 rA, rB, gA, gB;
  rA.a = rA.b = rB.a = rB.b = gA.a = gA.b = gB.a = gB.b = z4;
  if (b >= b1) return;
  rA = ld_stream32(R + 2 * (int64_t)b);
  gA = ld_keep32(nr + 2 * (int64_t)__ldg(v.nbr + b));
  int mB = b + L < b1 ? __ldg(v.nbr + b + L) : -1;
  int mA = -1;
  for (;;) {
    // bond b from set A; set B takes b + L
    int bn = b + L;
    if (bn < b1) {
      rB = ld_stream32(R + 2 * (int64_t)bn);
      gB = ld_keep32(nr + 2 * (int64_t)mB);
    }
    mA = __float_as_int(rA.b.z);            // neighbour of b + 2L
    bond3(v, R, b, rA, gA, c);
    b = bn;
    if (b >= b1) break;
    // bond b from set B; set A takes b + L
    bn = b + L;
    if (bn < b1) {
      rA = ld_stream32(R + 2 * (int64_t)bn);
      gA = ld_keep32(nr + 2 * (int64_t)mA);
    }
    mB = __float_as_int(rB.b.z);
    bond3(v, R, b, rB, gB, c);
    b = bn;
    if (b >= b1) break;
  }
}

template <int D, int L>
__device__ __forceinline__ void mixed_family_item(const StepArgs& a, const float* ke, int64_t t) {
  constexpr int RS = D == 3 ? 2 : 1;       // float4 per bond record
  const DevView& v = a.v;
  const float4* nr = a.uf_n;               // node records of u_n
  const LoadMixed<D> load_u{nr, v.dtv};
  const int item = (int)(t / L);
  const int lane = (int)(t % L);
  const bool valid = item < v.n_fam;
  const int f = valid ? v.fam_order[item] : 0;
  const int node = valid ? v.fam_node[f] : 0;
  float acc[D];
#pragma unroll
  for (int i = 0; i < D; i++) acc[i] = 0.f;
  int nbroken = 0;
  if (valid) {
    const int b0 = v.fam_ptr[f], b1 = v.fam_ptr[f + 1];
    const bool brk = a.mode >= 1 && v.fail3 && v.fam_intact[f] >= v.fam_brk[f];
    const float s0fam = D == 2 ? v.fam_s0f[f] : 0.f;     // 3D records carry their threshold
    const bool force = a.mode != 2;
    const int corr0 = v.fam_corr[f];
    const float4 xk = nr[2 * node];
    const float4 qk = nr[2 * node + 1];
    float uk[D];
    load_u(node, uk);
    float4* R = a.brec;
    bool deferred = false;
    int b = b0 + lane;
    const float4 z4 = make_float4(0, 0, 0, 0);
    float4 ra = z4, rb = z4, na = z4, nb = z4;
    if constexpr (D == 3) {
      Bond3Ctx c;
      c.xk = xk;
      c.qk = qk;
#pragma unroll
      for (int i = 0; i < 3; i++) { c.uk[i] = uk[i]; c.acc[i] = 0.f; }
      c.b0 = b0;
      c.corr0 = corr0;
      c.nbroken = 0;
      c.brk = brk;
      c.force = force;
      c.deferred = false;
      family_loop3<L>(v, R, nr, b, b1, c);
#pragma unroll
      for (int i = 0; i < 3; i++) acc[i] = c.acc[i];
      nbroken = c.nbroken;
      deferred = c.deferred;
      b = b1;
    }
    if (D == 2 && b < b1) load_record<D>(R, b, ra, rb);
    if (D == 2 && b + L < b1) load_record<D>(R, b + L, na, nb);
    int m = D == 2 && b < b1 ? __float_as_int(ra.w) : -1;
    Rec32 g;
    g.a = z4;
    g.b = z4;
    if (m >= 0) g = ld_keep32(nr + 2 * m);
    // 2D: two-stage pipeline per lane, records two bonds ahead and the next
    // neighbour's node record requested before the current bond is computed
    while (D == 2 && b < b1) {
      const int bn = b + L;
      float4 qa = z4, qb = z4;
      if (bn + L < b1) load_record<D>(R, bn + L, qa, qb);
      const int mn = bn < b1 ? __float_as_int(na.w) : -1;
      Rec32 gn;
      gn.a = z4;
      gn.b = z4;
      if (mn >= 0) gn = ld_keep32(nr + 2 * mn);
      if (m >= 0) {
        const float4 um = g.b;
        bool cut = false;
        if (brk) {
          const float4 xm = g.a;
          const float x0 = xm.x - xk.x, x1 = xm.y - xk.y, x2 = xm.z - xk.z;
          const float e0 = um.x - qk.x, e1 = um.y - qk.y, e2 = D == 3 ? um.z - qk.z : 0.f;
          const float lhs = 2.f * (x0 * e0 + x1 * e1 + x2 * e2) + (e0 * e0 + e1 * e1 + e2 * e2);
          float rhs;
          if (D == 3) {
            rhs = rb.w;     // s0b (2 + s0b) |xi|^2, from the record
          } else {
            const float sc = bond_s0_f32(s0fam, a.pertf, bond_hash(v.s0_seed32, node, m));
            rhs = sc * (2.f + sc) * (x0 * x0 + x1 * x1 + x2 * x2);
          }
          if (fabsf(lhs - rhs) <= 2e-4f * rhs) {
            // Near the threshold: decided in FP64 by the pass after the loop,
            // which also adds the bond's force if it stays intact.
            deferred = true;
            cut = true;
          } else if (lhs > rhs) {
            cut = true;
            mark_broken<D>(R, b, m, rhs);
            atomicAnd(&v.state[b >> 5], ~(1u << (b & 31)));
            nbroken++;
          }
        }
        if (force && !cut) {
          float du[D];
          du[0] = um.x;
          du[1] = um.y;
          if (D == 3) du[D - 1] = um.z;
          const unsigned fl = __float_as_uint(um.w);
          if (fl) {
#pragma unroll
            for (int i = 0; i < D; i++)
              if ((fl >> i) & 1u) du[i] += (float)v.dtv[3 * m + i];
          }
#pragma unroll
          for (int i = 0; i < D; i++) du[i] -= uk[i];
          bond_force<D>(ra, rb, du, acc);
          if (corr0 >= 0) corr_apply<D>(v, (int64_t)corr0 + (b - b0), du, acc);
        }
      }
      b = bn;
      ra = na;
      rb = nb;
      na = qa;
      nb = qb;
      m = mn;
      g = gn;
    }
    if (deferred) {
      // Rare: repeat the FP32 test on this lane's bonds and settle the ones
      // in the band with the reference's FP64 expression.
      for (b = b0 + lane; b < b1; b += L) {
        ra = R[(int64_t)RS * b];
        if (D == 3) rb = R[(int64_t)RS * b + 1];
        if (D == 3 ? !(rb.w > 0.f) : __float_as_int(ra.w) < 0) continue;
        const int m = D == 3 ? v.nbr[b] : __float_as_int(ra.w);
        const float4 xm = nr[2 * m], um = nr[2 * m + 1];
        const float x0 = xm.x - xk.x, x1 = xm.y - xk.y, x2 = xm.z - xk.z;
        const float e0 = um.x - qk.x, e1 = um.y - qk.y, e2 = D == 3 ? um.z - qk.z : 0.f;
        const float lhs = 2.f * (x0 * e0 + x1 * e1 + x2 * e2) + (e0 * e0 + e1 * e1 + e2 * e2);
        const uint32_t h = bond_hash(v.s0_seed32, node, m);
        float rhs;
        if (D == 3) {
          rhs = rb.w;
        } else {
          const float sc = bond_s0_f32(s0fam, a.pertf, h);
          rhs = sc * (2.f + sc) * (x0 * x0 + x1 * x1 + x2 * x2);
        }
        if (!(fabsf(lhs - rhs) <= 2e-4f * rhs)) continue;
        if (stretch_over_fp64<D>(v, a.u_n, node, m, bond_s0(v.fam_s0[f], v.s0_pert, h))) {
          mark_broken<D>(R, b, m, rhs);
          atomicAnd(&v.state[b >> 5], ~(1u << (b & 31)));
          nbroken++;
        } else if (force) {
          float du[D];
          load_u(m, du);
#pragma unroll
          for (int i = 0; i < D; i++) du[i] -= uk[i];
          bond_force<D>(ra, rb, du, acc);
          if (corr0 >= 0) corr_apply<D>(v, (int64_t)corr0 + (b - b0), du, acc);
        }
      }
    }
    if (force) {
      const int j0 = v.fe_adj_ptr[node], j1 = v.fe_adj_ptr[node + 1];
      for (int j = j0 + lane; j < j1; j += L) {
        const int ent = v.fe_adj[j];
        fe_rows<D, float>(v, ke, ent >> 3, ent & 7, load_u, acc);
      }
    }
  }
  warp_sum<D, L>(acc);
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) nbroken += __shfl_xor_sync(kFull, nbroken, o);
  if (lane == 0 && valid && nbroken) v.fam_intact[f] -= nbroken;
  if (a.mode == 2) return;
  if (lane == 0 && valid) external_force<D>(a, node, acc);
  warp_update<D, L, true>(a, acc, valid ? node : -1);
}

// 2D FE-only nodes of one lattice tile, one node per thread.  The tile's
// sites and a one-site halo are staged in shared memory as FP32
// displacements (the FP64 state rounded on the integer pipe, plus this
// step's increment for varying prescribed DOFs), so each staged value is
// read from HBM once per tile (1.27 times per node) instead of once per
// stencil neighbour; a site's node is the row's first node id plus the
// number of present sites before it.  The stencil runs over the 9 lattice
// offsets with the class's blocks (zero blocks where the class has no
// neighbour); the node is then updated in FP64 and its FP32 record is
// written only if the PD part of the step reads it.
__device__ __forceinline__ void tile_item2(const StepArgs& a, int tile, float2* su) {
  using T = Tile2;
  const DevView& v = a.v;
  const int2* rows = v.tile_rows + (int64_t)tile * T::ROWS;
  for (int q = threadIdx.x; q < T::SITES; q += blockDim.x) {
    const int r = q / T::WX, x = q - r * T::WX;
    const int2 ri = __ldg(rows + r);
    float2 w = make_float2(0.f, 0.f);
    if (((unsigned)ri.y >> x) & 1u) {
      const int n = ri.x + __popc((unsigned)ri.y & ((1u << x) - 1u));
      const unsigned fl = v.bcflag[n];
      double2 c = *reinterpret_cast<const double2*>(a.u_n + 2 * (int64_t)n);
      if (fl & 1u) c.x += v.dtv[3 * n];
      if (fl & 2u) c.y += v.dtv[3 * n + 1];
      w = make_float2(d2f_bits(c.x), d2f_bits(c.y));
    }
    su[q] = w;
  }
  const int x = threadIdx.x % T::X, y = threadIdx.x / T::X;
  const int ctr = (x + 1) + T::WX * (y + 1);
  const int cc = v.tile_cls[(int64_t)tile * T::NODES + threadIdx.x];
  int node = -1;
  if (cc >= 0) {
    const int2 ri = __ldg(rows + y + 1);
    node = ri.x + __popc((unsigned)ri.y & ((1u << (x + 1)) - 1u));
  }
  // update operands, requested before the barrier so their loads overlap the staging
  double2 un = make_double2(0.0, 0.0), prev = make_double2(0.0, 0.0);
  float dt2m = 0.f;
  unsigned fl = 0;
  if (node >= 0) {
    un = *reinterpret_cast<const double2*>(a.u_n + 2 * (int64_t)node);
    prev = *reinterpret_cast<const double2*>(a.u_next + 2 * (int64_t)node);
    dt2m = v.dt2m_f[node];
    fl = v.bcflag[node];
  }
  __syncthreads();
  if (node < 0) return;
  float acc[2] = {0.f, 0.f};
  const float4* B = reinterpret_cast<const float4*>(v.lat_blk) + (int64_t)(cc & kTileClsMask) * T::SLOTS;
#pragma unroll
  for (int o = 0; o < T::SLOTS; o++) {
    const float4 b = __ldg(B + o);
    const float2 u = su[ctr + (o % 3 - 1) + T::WX * (o / 3 - 1)];
    acc[0] -= b.x * u.x + b.y * u.y;
    acc[1] -= b.z * u.x + b.w * u.y;
  }
  external_force<2>(a, node, acc);
  const double uo[2] = {un.x, un.y}, up[2] = {prev.x, prev.y};
  double unew[2];
#pragma unroll
  for (int i = 0; i < 2; i++) {
    if (!((fl >> (4 + i)) & 1u)) {
      const float tA = acc[i] * dt2m;
      unew[i] = a.mode == 0 ? uo[i] + f2d_bits(0.5f * tA) : fma(2.0, uo[i], -up[i]) + f2d_bits(tA);
    } else {
      unew[i] = (fl >> i) & 1u ? uo[i] + v.dtv[3 * node + i] : uo[i];
    }
  }
  *reinterpret_cast<double2*>(a.u_next + 2 * (int64_t)node) = make_double2(unew[0], unew[1]);
  if (cc & kTileShadowBit)
    a.uf_next[2 * (int64_t)node + 1] = make_float4(d2f_bits(unew[0]), d2f_bits(unew[1]), 0.f, __uint_as_float(fl));
}

// Blocks per SM: 4 in 3D (64 registers: the two-stage family pipeline holds
// two bond records and a node record per lane; C2 47.0 us per step against
// 48.5 with 5 blocks); 6 in 2D (40 registers, a few spills to L1), which took
// the 256-plate batch from 700 to 564 us per step (the 2D step waits on its
// gathers; more resident warps hide more of them).
template <int D, int LP, int LF>
__global__ void __launch_bounds__(256, D == 3 ? 4 : 6) k_step_mixed(StepArgs a) {
  extern __shared__ __align__(16) float s_ke[];
  const float* ke = a.v.ke32;
  if (a.ke_smem) {
    for (int i = threadIdx.x; i < a.ke_smem; i += blockDim.x) s_ke[i] = a.v.ke32[i];
    __syncthreads();
    ke = s_ke;
  }
  if ((int)blockIdx.x < a.pd_blocks) {
    mixed_family_item<D, LP>(a, ke, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
  } else if (D == 2 && a.v.n_tiles > 0) {
    const int tb = (int)blockIdx.x - a.pd_blocks;
    if (tb < a.v.n_tiles) {
      __shared__ float2 s_tile[Tile2::SITES];
      tile_item2(a, tb, s_tile);
    } else {
      const int64_t t = (int64_t)(tb - a.v.n_tiles) * blockDim.x + threadIdx.x;
      feonly_item<D, LF, float, true>(a, ke, t, LoadMixed<D>{a.uf_n, a.v.dtv}, a.v.fe_rest, a.v.n_rest);
    }
  } else {
    const int64_t t = (int64_t)(blockIdx.x - a.pd_blocks) * blockDim.x + threadIdx.x;
    feonly_item<D, LF, float, true>(a, ke, t, LoadMixed<D>{a.uf_n, a.v.dtv});
  }
}

// Mixed-precision bond records from the FP32 coefficients, the bond states and
// the per-bond thresholds.
template <int D>
__global__ void k_pack_bonds(DevView v, float pertf, int lanes, float4* rec) {
  const int f = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (f >= v.n_fam) return;
  const int k = v.fam_node[f];
  const int64_t nb = v.n_bond;
  const int b1 = v.fam_ptr[f + 1];
  for (int b = v.fam_ptr[f] + (threadIdx.x & 31); b < b1; b += 32) {
    const int m = v.nbr[b];
    const bool intact = (v.state[b >> 5] >> (b & 31)) & 1u;
    const int mb = intact ? m : ~m;
    if (D == 2) {
      rec[b] = make_float4(v.coef32[b], v.coef32[nb + b], v.coef32[2 * nb + b], __int_as_float(mb));
    } else {
      // threshold of the sqrt-free stretch test, s0b (2 + s0b) |xi|^2, from the FP32 positions
      const float s0b = bond_s0_f32(v.fam_s0f[f], pertf, bond_hash(v.s0_seed32, k, m));
      const float4 xk = v.Xf[k], xm = v.Xf[m];
      const float x0 = xm.x - xk.x, x1 = xm.y - xk.y, x2 = xm.z - xk.z;
      const float thr = s0b * (2.f + s0b) * (x0 * x0 + x1 * x1 + x2 * x2);
      const int ahead = b + 2 * lanes < b1 ? v.nbr[b + 2 * lanes] : -1;
      rec[2 * (int64_t)b] = make_float4(v.coef32[b], v.coef32[nb + b], v.coef32[2 * nb + b], v.coef32[3 * nb + b]);
      rec[2 * (int64_t)b + 1] =
          make_float4(v.coef32[4 * nb + b], v.coef32[5 * nb + b], __int_as_float(ahead), intact ? thr : -thr);
    }
  }
}

template <int D, int LP>
cudaError_t mixed_dispatch_lf(const StepArgs& a, int lf, int blocks, size_t smem, cudaStream_t s) {
  switch (lf) {
    case 1: k_step_mixed<D, LP, 1><<<blocks, 256, smem, s>>>(a); break;
    case 2: k_step_mixed<D, LP, 2><<<blocks, 256, smem, s>>>(a); break;
    case 4: k_step_mixed<D, LP, 4><<<blocks, 256, smem, s>>>(a); break;
    case 8: k_step_mixed<D, LP, 8><<<blocks, 256, smem, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <int D>
cudaError_t mixed_dispatch(StepArgs a, int lp, int lf, cudaStream_t s) {
  const int pd_blocks = (int)(((int64_t)a.v.n_fam * lp + 255) / 256);
  const int fe_blocks = a.mode == 2 ? 0
                        : D == 2 && a.v.n_tiles > 0 ? a.v.n_tiles + (int)(((int64_t)a.v.n_rest * lf + 255) / 256)
                                                    : (int)(((int64_t)a.v.n_feonly * lf + 255) / 256);
  a.pd_blocks = pd_blocks;
  const int blocks = pd_blocks + fe_blocks;
  if (blocks == 0) return cudaSuccess;
  const size_t smem = (size_t)a.ke_smem * sizeof(float);
  switch (lp) {
    case 4: return mixed_dispatch_lf<D, 4>(a, lf, blocks, smem, s);
    case 8: return mixed_dispatch_lf<D, 8>(a, lf, blocks, smem, s);
    case 16: return mixed_dispatch_lf<D, 16>(a, lf, blocks, smem, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t launch_step_mixed(const StepArgs& a, int lp, int lf, cudaStream_t s) {
  return a.v.dim == 2 ? mixed_dispatch<2>(a, lp, lf, s) : mixed_dispatch<3>(a, lp, lf, s);
}

cudaError_t launch_pack_bonds(const DevView& v, float pertf, int lanes, float4* rec, cudaStream_t s) {
  if (v.n_fam == 0) return cudaSuccess;
  const int blocks = (v.n_fam + 7) / 8;
  if (v.dim == 2) k_pack_bonds<2><<<blocks, 256, 0, s>>>(v, pertf, lanes, rec);
  else k_pack_bonds<3><<<blocks, 256, 0, s>>>(v, pertf, lanes, rec);
  return cudaGetLastError();
}

}  // namespace pdx
