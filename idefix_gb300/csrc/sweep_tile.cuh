// FP32 y and z sweeps of 3-D blocks over tiles staged by the tensor-memory
// accelerator (mixed-precision path).
#pragma once
#include <cuda.h>

#include "mhd_kernels.cuh"

namespace idfx {

// ---------------------------------------------------------------------------
// A CTA owns kTX x-columns by kTB rows of the other transverse direction
// (lane l of warp w: column x0 + l % 16, row 2 w + l / 16) and marches a
// segment of cells along the sweep direction, as the per-thread march does,
// with the same arithmetic lane for lane: reconstruction of every cell once,
// one Riemann problem per face, the flux difference into Uc, the face EMFs,
// InvDt.  What differs is where the operands come from: the cells of the
// tile at one position along the sweep (a "slab": the FP32 primitives of
// every variable, the FP64 conserved hydro state and, when InvDt is
// accumulated, InvDt) arrive in a ring of shared-memory slots by
// cp.async.bulk.tensor copies of 4-D boxes (x, y, z, variable), one mbarrier
// per slot.  A lane reads its whole stencil and its conserved state from the
// ring, so the march's register window and register prefetch disappear.
// Every warp releases a slab after its last use (an acquire-release counter
// per slot); the warp that releases it last issues the copy of the slab
// that takes its slot, so no warp waits for a producer.  Waits are bounded:
// on a timeout the stage reports a CUDA-side error and stops the cycle.
// Needs nt0 a multiple of 4 and 16-byte aligned arrays (tensor-map strides
// and box origins), and reconstruction orders 2-4; the march runs otherwise.
// ---------------------------------------------------------------------------
constexpr int kTX = 16;    // x columns of a tile (the box origin x0 = 16 bx is 16-byte aligned)
constexpr int kTB = 8;     // rows of the other transverse direction
constexpr int kTW = 4;     // warps per CTA (two rows each)
constexpr int kTLook = 1;  // slabs in flight beyond the stencil

constexpr int kTSlabV = 8 * kTB * kTX * 4;  // FP32 primitives [NV = 8][kTB][kTX]
constexpr int kTSlabU = 5 * kTB * kTX * 8;  // FP64 hydro state [5][kTB][kTX]
constexpr int kTSlabI = kTB * kTX * 8;      // FP64 InvDt [kTB][kTX]
constexpr int kTSlab = kTSlabV + kTSlabU + kTSlabI;
static_assert(kTSlabV % 128 == 0 && kTSlabU % 128 == 0 && kTSlab % 128 == 0, "slab parts 128-byte aligned");

template <int ORDER>
__host__ __device__ constexpr int tile_ring() {
  return 2 * Recon<ORDER>::H + 1 + kTLook;
}
// ring slots, then the mbarriers and the release counters of the slots
template <int ORDER>
__host__ __device__ constexpr int tile_smem() {
  return tile_ring<ORDER>() * kTSlab + 128;
}
static_assert(tile_ring<4>() * 12 <= 128, "barriers and counters fit their 128 bytes");

// tensor maps of the FP32 primitives, the conserved state and InvDt, with
// the box of the y sweep ([0]) and of the z sweep ([1])
struct SweepTileMaps {
  CUtensorMap vc[2], uc[2], inv[2];
};

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* tm, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, int c0, int c1, int c2, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.cta.shared::cta.add.u32 %0, [%1], %2;" : "=r"(old) : "r"(smem_u32(p)), "r"(v) : "memory");
  return old;
}

template <int DIR, int ORDER, int SOLVER>
__global__ void __launch_bounds__(32 * kTW) k_sweep_tile(Geo g, Fields f, const Ctl* ctl, int invdt, int last_dir,
                                                        int seg, const __grid_constant__ CUtensorMap tmv,
                                                        const __grid_constant__ CUtensorMap tmu,
                                                        const __grid_constant__ CUtensorMap tmi) {
  constexpr int D = 3;
  using T = float;
  using v = Var<D>;
  using dd = Dir<D, DIR>;
  constexpr int NV = v::NV;
  constexpr int NU = v::BX1;
  constexpr int H = Recon<ORDER>::H;
  constexpr int R = tile_ring<ORDER>();
  constexpr int B = (DIR == 2) ? 1 : 2;  // the other transverse direction
  static_assert(DIR == 1 || DIR == 2, "tile sweep: y and z");
  static_assert(H >= 1, "tile sweep: reconstruction orders 2-4");
  static_assert(NV == 8 && NU == 5, "slab layout of a 3-D block");
  extern __shared__ __align__(128) unsigned char tsm[];
  if (ctl->done) return;
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  uint64_t* full = reinterpret_cast<uint64_t*>(tsm + R * kTSlab);
  unsigned* cnt = reinterpret_cast<unsigned*>(tsm + R * kTSlab + 8 * R);
  const int xl = lane & (kTX - 1), br = 2 * w + (lane >> 4);
  const int x0 = (int)blockIdx.x * kTX;
  const int b0 = g.beg[B] - g.ext + (int)blockIdx.y * kTB;
  const int x = x0 + xl, b = b0 + br;
  // columns of the sweep: the active ones and the CT extension around them
  const bool col = x >= g.beg[0] - g.ext && x < g.end[0] + g.ext && b < g.end[B] + g.ext;
  const bool active = col && x >= g.beg[0] && x < g.end[0] && b >= g.beg[B] && b < g.end[B];
  const int m0 = g.beg[DIR] + (int)blockIdx.z * seg;
  const int m1 = min(m0 + seg, g.end[DIR]);
  const int mlo = m0 - 1 - H;             // position of slab 0 along the sweep
  const int nslab = m1 - m0 + 2 * H + 2;  // slabs mlo .. m1 + H
  const int nstep = m1 - m0 + 2;          // steps: cells m0 - 1 .. m1
  const uint32_t slab_bytes = kTSlabV + kTSlabU + (invdt == 2 ? kTSlabI : 0);
  // one thread: slab q into slot q % R (box origins: x0, the row, the slab)
  auto issue = [&](int q) {
    unsigned char* dst = tsm + (q % R) * kTSlab;
    uint64_t* bar = full + (q % R);
    const int m = mlo + q;
    const int cy = (DIR == 1) ? m : b0, cz = (DIR == 1) ? b0 : m;
    mbar_expect(bar, slab_bytes);
    tma_load_4d(dst, &tmv, x0, cy, cz, 0, bar);
    tma_load_4d(dst + kTSlabV, &tmu, x0, cy, cz, 0, bar);
    if (invdt == 2) tma_load_3d(dst + kTSlabV + kTSlabU, &tmi, x0, cy, cz, bar);
  };
  if (threadIdx.x == 0) {
    for (int s = 0; s < R; s++) {
      mbar_init(full + s);
      cnt[s] = 0u;
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int q = 0; q < min(R, nslab); q++) issue(q);
  }
  __syncthreads();
  auto V = [&](int q, int n) -> T {
    return reinterpret_cast<const float*>(tsm + (q % R) * kTSlab)[(n * kTB + br) * kTX + xl];
  };
  auto U = [&](int q, int n) -> double {
    return reinterpret_cast<const double*>(tsm + (q % R) * kTSlab + kTSlabV)[(n * kTB + br) * kTX + xl];
  };
  auto I = [&](int q) -> double {
    return reinterpret_cast<const double*>(tsm + (q % R) * kTSlab + kTSlabV + kTSlabU)[br * kTX + xl];
  };
  int idx[3];
  idx[0] = x;
  idx[DIR] = m0;
  idx[B] = b;
  const long long c0 = cidx(g, idx[2], idx[1], idx[0]);  // cell m0 of this column
  const long long f0 = fidx(g, idx[2], idx[1], idx[0]);
  const long long sd = g.s[DIR], fsd = g.fs[DIR];
  const double* vs = f.Vs + DIR * g.nface;
  const T gam = (T)g.gamma;
  const T dxd = (T)g.dx[DIR];
  const Recip l3{g.l3b[DIR], g.l3y[DIR]};
  const T dtdVT = (T)ctl->dtdV;
  const T areaT = (T)g.A[DIR];
  const T invdxT = T(1) / (T)g.dx[DIR];
  T vrp[NV];     // right-face state of the previous cell
  T Fp[NU];      // flux x area of the previous face
  T cp = T(0);   // cmax of the previous face
#pragma unroll
  for (int n = 0; n < NV; n++) vrp[n] = T(0);
#pragma unroll
  for (int n = 0; n < NU; n++) Fp[n] = T(0);
  double nbn = col ? vs[f0] : 0.0;  // normal face field of the next face (face m0)
  double run_max = 0.0;
  int waited = -1;  // slabs 0 .. waited have landed
  bool ok = true;
  for (int s = 0; s < nstep; s++) {
    const int c = m0 - 1 + s;
    // the stencil of cell c: slabs s .. s + 2H; the state of cell c - 1: slab s - 1 + H
    const int need = min(s + 2 * H, nslab - 1);
    while (ok && waited < need) {
      const int q = waited + 1;
      ok = mbar_wait(full + (q % R), (uint32_t)((q / R) & 1));
      if (ok) waited = q;
    }
    ok = __all_sync(0xffffffffu, ok);  // the warp stops together
    if (!ok) break;
    if (col) {
      const long long cc = c0 + (long long)(c - m0) * sd;
      T vl[NV], vr[NV];
      const bool shk = f.shock && f.shock[cc];
#pragma unroll
      for (int n = 0; n < NV; n++) {
        if (n == dd::BXn) continue;
        T wv[2 * H + 1];
#pragma unroll
        for (int m = 0; m <= 2 * H; m++) wv[m] = V(s + m, n);
        Recon<ORDER>::cell(wv, dxd, n == v::RHO || n == v::PRS, vl[n], vr[n], shk, l3);
      }
      if (s >= 1) {
        T vL[NV], vR[NV];
#pragma unroll
        for (int n = 0; n < NV; n++) {
          if (n == dd::BXn) continue;
          vL[n] = vrp[n];
          vR[n] = vl[n];
        }
        const T bn = from_f64<T>(nbn);
        if (s + 1 < nstep) nbn = vs[f0 + (long long)(c + 1 - m0) * fsd];
        vL[dd::BXn] = bn;
        vR[dd::BXn] = bn;
        RiemannOut<D, T> r;
        riemann<D, DIR, SOLVER>(gam, (T)g.rgm1, vL, vR, r);
        store_emf<D, DIR>(g, f, cc, r, vL, vR);
        if (active) {
          T FA[NU];
#pragma unroll
          for (int n = 0; n < NU; n++) FA[n] = r.F[n] * areaT;
          if (s >= 2) {  // cell c - 1
            const long long cu = cc - sd;
            const int qu = s - 1 + H;
#pragma unroll
            for (int n = 0; n < NU; n++) {
              const T rhs = -dtdVT * (FA[n] - Fp[n]);
              f.Uc[n * g.ncell + cu] = U(qu, n) + to_f64(rhs);
            }
            if (invdt) {
              const double prev = (invdt == 1) ? 0.0 : I(qu);
              const double inv = prev + to_f64(T(0.5) * (r.cmax + cp) * invdxT);
              f.InvDt[cu] = inv;
              if (inv > run_max) run_max = inv;  // NaN never compares greater
            }
          }
#pragma unroll
          for (int n = 0; n < NU; n++) Fp[n] = FA[n];
          cp = r.cmax;
        }
      }
#pragma unroll
      for (int n = 0; n < NV; n++) vrp[n] = vr[n];
    }
    // slab s is read for the last time: the last warp to release it fetches
    // slab s + R into its slot
    __syncwarp();
    if (lane == 0) {
      const unsigned old = atom_add_acq_rel(cnt + (s % R), 1u);
      if ((old & (kTW - 1)) == kTW - 1 && s + R < nslab) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue(s + R);
      }
    }
  }
  if (!ok) {
    // a copy did not land: stop the cycle; wait (bounded) for the copies
    // that may still be in flight before the shared memory is released
    if (lane == 0) report_wait_timeout(ctl);
    for (int q = waited + 1; q < min(nslab, waited + 1 + R); q++)
      mbar_wait(full + (q % R), (uint32_t)((q / R) & 1));
    __syncwarp();
    return;
  }
  if (last_dir && invdt && active) atomic_max_pos((unsigned long long*)&((Ctl*)ctl)->invdt_max_bits, run_max);
}

}  // namespace idfx
