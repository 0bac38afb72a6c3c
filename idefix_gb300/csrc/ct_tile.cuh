// Corner EMFs fused with the face update over tiles whose EMF inputs are
// staged by the tensor-memory accelerator (mixed-precision path, 3-D
// periodic blocks; uct_contact, arithmetic and uct0).
#pragma once
#include <cuda.h>

#include "sweep_tile.cuh"

namespace idfx {

// ---------------------------------------------------------------------------
// The tiling and the arithmetic are k_ct_fused's: a CTA owns 32 x 8 edge
// columns (plus the +i column and +j row beyond them) and marches a segment
// of layers, computing each layer's corner EMFs into a shared-memory plane and
// updating the faces of the layer below from it.  What differs is where the
// corner EMFs' inputs come from: the twelve FP32 EMF arrays (face EMFs, upwind
// weights, cell EMFs - consecutive arrays of a block's pool) of one layer,
// over x from a 16-byte aligned start at or below i0 - 1 through i0 + 32 and
// y from j0 - 1 through j0 + 8, arrive as one 4-D box (x, y, z, array) of a
// tensor map in a ring of three layer slots, one mbarrier per slot.  The
// corners of layer k + 1 read layers k and k + 1 from the ring; when they
// start, the copy of layer k + 2 is already in flight into the slot that
// layer k - 1 left.  The faces themselves are read and written in global
// memory (their rows of nt0 + 1 doubles are not 16-byte strided), with an L2
// prefetch two layers ahead.  Waits are bounded; a CTA whose wait gives up
// sets the error status, stops with its whole block at the next layer
// barrier and waits (bounded) for its copies in flight before it exits.
// ---------------------------------------------------------------------------
constexpr int kCsX = 40;                         // staged x extent (i0 - 1 .. i0 + 32 from an aligned start)
constexpr int kCsY = kCtTJ + 2;                  // j0 - 1 .. j0 + kCtTJ
constexpr int kCsRing = 3;                       // layer slots
constexpr int kCsSlab = kEaN * kCsY * kCsX * 4;  // bytes of one staged layer
static_assert(kCsSlab % 128 == 0, "layer slots 128-byte aligned");
static_assert((kCsX * 4) % 16 == 0, "box inner extent a multiple of 16 bytes");

// the tensor map of the twelve EMF arrays of a block (engine.cu: ct_tile_map)
struct CtTileMap {
  CUtensorMap emf;
};

__host__ __device__ constexpr int ct_tile_planes_off() { return kCsRing * kCsSlab; }
__host__ __device__ constexpr int ct_tile_bar_off() {
  return (ct_tile_planes_off() + (int)sizeof(CtPlanes<float>) + 7) / 8 * 8;
}
__host__ __device__ constexpr int ct_tile_smem() { return ct_tile_bar_off() + 8 * kCsRing; }

__global__ void __launch_bounds__(kCtTI * kCtTJ, 3) k_ct_tile(Geo g, Fields f, const Ctl* ctl, int combine, double wc,
                                                          double w0, const __grid_constant__ CUtensorMap tm) {
  constexpr int D = 3;
  using E = float;
  extern __shared__ __align__(128) unsigned char csm[];
  if (ctl->done) return;
  float* ring = reinterpret_cast<float*>(csm);
  CtPlanes<E>& P = *reinterpret_cast<CtPlanes<E>*>(csm + ct_tile_planes_off());
  uint64_t* bar = reinterpret_cast<uint64_t*>(csm + ct_tile_bar_off());
  CtPos p;
  p.ti = threadIdx.x;
  p.tj = threadIdx.y;
  const int i0 = g.beg[0] + (int)blockIdx.x * kCtTI, j0 = g.beg[1] + (int)blockIdx.y * kCtTJ;
  p.i = i0 + p.ti;
  p.j = j0 + p.tj;
  const int ie = g.end[0], je = g.end[1], ke = g.end[2];  // edge positions run over [beg, end]
  p.own = p.i <= ie && p.j <= je;
  p.hkind = (p.tj == 0) ? 1 : (p.tj == 1 && p.ti < kCtTJ) ? 2 : 0;
  p.hi = (p.hkind == 1) ? p.i : i0 + kCtTI;
  p.hj = (p.hkind == 1) ? j0 + kCtTJ : j0 + p.ti;
  p.halo = p.hkind != 0 && p.hi <= ie && p.hj <= je;
  const int i = p.i, j = p.j, ti = p.ti, tj = p.tj;
  const int x0 = (i0 - 1) & ~3, y0 = j0 - 1;  // box origin (x: 16-byte aligned)
  const int k0 = g.beg[2] + (int)blockIdx.z * kCtKSeg;
  const int k1 = min(k0 + kCtKSeg, ke + 1);  // face layers k0 .. k1-1
  const int kmax = min(k1, ke);               // last layer whose corners are computed
  const bool lead = threadIdx.x == 0 && threadIdx.y == 0;
  // layer L lives in slot (L - k0 + 1) % kCsRing; its copy completes phase
  // ((L - k0 + 1) / kCsRing) & 1 of that slot's barrier
  auto slot = [&](int L) { return (L - k0 + 1) % kCsRing; };
  auto phase = [&](int L) { return (uint32_t)(((L - k0 + 1) / kCsRing) & 1); };
  auto issue = [&](int L) {
    uint64_t* b = bar + slot(L);
    mbar_expect(b, (uint32_t)kCsSlab);
    tma_load_4d(csm + slot(L) * kCsSlab, &tm, x0, y0, L, 0, b);
  };
  int issued = k0 - 2;  // layers k0 - 1 .. issued are in flight or landed
  if (lead) {
    for (int s = 0; s < kCsRing; s++) mbar_init(bar + s);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // the first three layers; every thread counts what the lead thread issued
  for (int L = k0 - 1; L <= min(k0 + 1, kmax); L++) {
    if (lead) issue(L);
    issued = L;
  }
  bool ok = true;
  auto S = [&](int L) { return ring + slot(L) * (kCsSlab / 4); };
  // corner EMFs of layer L at edge (ei, ej) from the ring (layers L, L - 1)
  auto corners = [&](int L, int ei, int ej, int mask_kind, E& ox, E& oy, E& oz) {
    const float* s0 = S(L);
    const float* s1 = S(L - 1);
    auto get = [&](int q, int di, int dj, int dk) -> E {
      return (dk ? s1 : s0)[(q * kCsY + (ej + dj - y0)) * kCsX + (ei + di - x0)];
    };
    if (mask_kind == 0) corner_emfs_avg<D, E, kCxyz>(g.emf, get, ox, oy, oz);
    else if (mask_kind == 1) corner_emfs_avg<D, E, kCz | kCx>(g.emf, get, ox, oy, oz);
    else corner_emfs_avg<D, E, kCz | kCy>(g.emf, get, ox, oy, oz);
  };
  auto layer = [&](int L, int b, E& ox, E& oy, E& oz) {
    if (p.own) {
      corners(L, i, j, 0, ox, oy, oz);
      P.z[b][tj][ti] = oz;
      P.y[b][tj][ti] = oy;
      P.x[b][tj][ti] = ox;
    }
    if (p.halo) {
      E hx = E(0), hy = E(0), hz = E(0);
      if (p.hkind == 1) {
        corners(L, p.hi, p.hj, 1, hx, hy, hz);
        P.z[b][kCtTJ][ti] = hz;
        P.x[b][kCtTJ][ti] = hx;
      } else {
        corners(L, p.hi, p.hj, 2, hx, hy, hz);
        P.z[b][ti][kCtTI] = hz;
        P.y[b][ti][kCtTI] = hy;
      }
    }
  };
  E cx = E(0), cy = E(0), cz = E(0);  // own corner EMFs of layer k
  ok = mbar_wait(bar + slot(k0 - 1), phase(k0 - 1)) && mbar_wait(bar + slot(k0), phase(k0));
  if (ok) layer(k0, 0, cx, cy, cz);
  bool stop = __syncthreads_or(!ok);
  for (int k = k0; k < k1 && !stop; k++) {
    const int b = (k - k0) & 1;
    // layer k - 1 is read no more: its slot takes layer k + 2
    if (k + 2 <= kmax) {
      if (lead) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue(k + 2);
      }
      issued = k + 2;
    }
    if (k + 2 <= ke) {  // the faces two layers ahead, into L2
      const bool f0 = (combine & (kCtCombine | kCtSaveBegin)) != 0;
      if (p.own && (threadIdx.x & 7) == 0) {
        const long long fq = fidx(g, k + 2, j, i);
#pragma unroll
        for (int d = 0; d < 3; d++) {
          prefetch_l2(f.Vs + d * g.nface + fq);
          prefetch_l2(f.Vs + d * g.nface + fq + 4);
          if (f0) {
            prefetch_l2(f.Vs0 + d * g.nface + fq);
            prefetch_l2(f.Vs0 + d * g.nface + fq + 4);
          }
        }
      }
    }
    E nx = E(0), ny = E(0), nz = E(0);  // own corner EMFs of layer k + 1
    if (k + 1 <= ke) {
      ok = mbar_wait(bar + slot(k + 1), phase(k + 1));
      if (ok) layer(k + 1, b ^ 1, nx, ny, nz);
    }
    if (ok && p.own) {
      const bool in_i = i < ie, in_j = j < je, in_k = k < ke;
      faces_from_corners<D, E>(g, f, ctl, fidx(g, k, j, i), in_i, in_j, in_k, combine, wc, w0,
                               [&](int comp, int o) -> E {
                                 if (comp == 2) return o == 0 ? cz : (o == 1 ? P.z[b][tj][ti + 1] : P.z[b][tj + 1][ti]);
                                 if (comp == 1) return o == 0 ? cy : (o == 1 ? P.y[b][tj][ti + 1] : ny);
                                 return o == 0 ? cx : (o == 2 ? P.x[b][tj + 1][ti] : nx);
                               });
    }
    cx = nx;
    cy = ny;
    cz = nz;
    stop = __syncthreads_or(!ok);
  }
  if (stop) {
    // a copy did not land: stop the cycle; wait (bounded) for every copy
    // issued before the shared memory is released
    if (lead) report_wait_timeout(ctl);
    // (the last kCsRing layers issued: each still owns its slot's latest phase)
    for (int L = max(k0 - 1, issued - kCsRing + 1); L <= issued; L++) mbar_wait(bar + slot(L), phase(L));
  }
}

}  // namespace idfx
