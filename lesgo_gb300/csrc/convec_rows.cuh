// The convective term's x-rows on the 3/2 grid in one pass (convec.f90:
// 170-255): c2r of the six padded spectra of a row (u, v, w and the three
// vorticity components after the y pass with 3/2 padding), the three
// dealiased products at each level, and the r2c of the products, keeping
// the nx/2 modes that the truncation back to the small grid keeps.  The
// 3/2-grid fields never go to HBM: a block owns `rt` rows of one instance
// and a chunk of levels, and marches up the chunk with the c2r results of
// the levels k-1, k and k+1 held in shared memory (the products at level k
// read w and the vorticity at k+1 and u, v at k-1).  The spectra of the
// next level arrive by a bulk copy issued as soon as the current level's
// have been read, so it runs under the current level's transforms.
#pragma once
#include "bulk_copy.cuh"
#include "fft_core.cuh"

namespace lesgo {

struct ConvRowsGeom {
  int M;          // real row length on the 3/2 grid (nx2)
  int K;          // modes present in the input and kept in the output (nx/2)
  int ny2;        // rows per level
  int nz;         // levels per instance (1..nz)
  int rt;         // rows per block
  int cz;         // levels per block (the chunk)
  int ls;         // shared line stride in complex elements (M/2 + 1)
  long long in_fs, out_fs;   // complex elements between fields
  FastDiv fH, fK, f2, f3, f6, frt;   // by M/2, K, 2 rt, 3 rt, 6 rt, rt
  int* err;       // set to 1 when a copy wait gives up
};

// Shared memory of a block, in complex elements: three level slots of 6 rt
// lines (the c2r results), one scratch of 6 rt lines (the other buffer of
// each c2r, then the two buffers of the products' r2c), and the staging
// buffer of the raw spectra of a level (6 fields x rt rows x K modes) that
// the bulk copies fill; the copy barrier follows.
__host__ __device__ inline long long conv_rows_stage_elems(int rt, int K) { return 6LL * rt * K; }
__host__ __device__ inline long long conv_rows_smem_elems(int rt, int ls, int K) {
  return 4LL * 6 * rt * ls + conv_rows_stage_elems(rt, K);
}

// R is the transforms' arithmetic type; the products are formed in it too.
template <typename R>
__global__ void __launch_bounds__(256) k_convec_rows(ConvRowsGeom g, FftPlan<R> plan, const cplx<R>* __restrict__ in,
                                                     cplx<R>* __restrict__ out, R c) {
  using T2 = cplx<R>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* base = reinterpret_cast<T2*>(smem_raw);
  const int H = g.M / 2;
  const int rt = g.rt;
  const int nl3 = 3 * rt;
  const long long slot_elems = 6LL * rt * g.ls;
  T2* S = base + 3 * slot_elems;   // scratch
  T2* stage = S + slot_elems;
  uint64_t* bar = reinterpret_cast<uint64_t*>(stage + conv_rows_stage_elems(rt, g.K));
  const int row0 = blockIdx.x * rt;
  const int rows = min(rt, g.ny2 - row0);
  const int inst = blockIdx.z;
  const int k0 = 1 + blockIdx.y * g.cz;
  const int k1 = min(k0 + g.cz, g.nz + 1);   // levels k0 .. k1-1
  auto slot_z = [&](int lev) { return reinterpret_cast<const R*>(base + (lev % 3) * slot_elems); };
  // the products at level k read level k+1 at the wall level and in the
  // interior (convec.f90:176-200); the level below the lid reads level k only
  auto needs_next = [&](int k) { return k <= g.nz - 1 && (k == 1 || k <= g.nz - 2); };

  // The block's c2r sequence, in order: entry e = (level, first field,
  // fields).  The level below the chunk is read for u and v only (fields 0,
  // 1), the level above it for w and the vorticity x, y (fields 2..4).
  // needs_next holds for a leading run of levels, so the entries after the
  // first ones are the consecutive levels k0 + 1, k0 + 2, ...
  const int e_lo = (k0 >= 2 && k0 <= g.nz - 1) ? 1 : 0;
  const int e_k0 = (k0 <= g.nz - 1) ? 1 : 0;
  auto entry = [&](int e, int& lev, int& f0, int& nf) {
    if (e < e_lo) { lev = k0 - 1; f0 = 0; nf = 2; return; }
    if (e < e_lo + e_k0) { lev = k0; f0 = 0; nf = 6; return; }
    lev = k0 + (e - e_lo - e_k0) + 1;
    if (lev < k1) { f0 = 0; nf = 6; } else { f0 = 2; nf = 3; }
  };
  int n_entries = e_lo + e_k0;
  for (int k = k0; k < k1; ++k) n_entries += needs_next(k) ? 1 : 0;

  // thread 0 arms the barrier for entry e (its phase e) and copies the
  // entry's rows' spectra (one contiguous run of rows x K modes per field)
  // into the staging buffer
  auto prefetch = [&](int e) {
    if (threadIdx.x != 0 || e >= n_entries) return;
    int lev, f0, nf;
    entry(e, lev, f0, nf);
    const unsigned bytes = (unsigned)(rows * g.K * sizeof(T2));
    const long long lrow = ((long long)inst * g.nz + (lev - 1)) * g.ny2 + row0;
    mbar_arrive_expect_tx(bar, bytes * nf);
    for (int f = 0; f < nf; ++f)
      bulk_g2s(stage + (long long)(f0 + f) * rt * g.K, in + (long long)(f0 + f) * g.in_fs + lrow * g.K, bytes, bar);
  };

  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_init_fence();
  }
  __syncthreads();
  prefetch(0);

  // c2r of entry e into slot lev % 3.  The load goes to the buffer from
  // which the stages end in the slot: the slot itself for an even stage
  // count, else the scratch.  Returns false if the copy wait gave up.
  auto c2r_entry = [&](int e) -> bool {
    int lev, f0, nf;
    entry(e, lev, f0, nf);
    const bool ok = mbar_wait(bar, (unsigned)(e & 1));
    if (__syncthreads_or(!ok)) return false;
    // by value: a reference into the parameter block chosen at run time
    // would make the compiler copy the block to local memory
    const FastDiv fnl = nf == 6 ? g.f6 : nf == 3 ? g.f3 : g.f2;
    T2* X = base + (lev % 3) * slot_elems + (long long)f0 * rt * g.ls;
    T2* Sx = S + (long long)f0 * rt * g.ls;
    T2* A = (plan.nf & 1) ? Sx : X;
    T2* B = (plan.nf & 1) ? X : Sx;
    const int nl = nf * rt;
    const T2* stg = stage + (long long)f0 * rt * g.K;
    for (int t = threadIdx.x; t < nl * H; t += blockDim.x) {
      const int l = g.fH.div(t), k = t - l * H;   // l = field offset * rt + row
      T2 z = czero<T2>();
      if (l - g.frt.div(l) * rt < rows) {
        const T2* src = stg + (long long)l * g.K;
        const T2 xk = k < g.K ? src[k] : czero<T2>();
        const int km = H - k;
        const T2 xm = (k > 0 && km < g.K) ? src[km] : czero<T2>();
        const T2 a = cadd_conj(xk, xm);
        const T2 b = csub_conj(xk, xm);
        const T2 w = ldt(plan.rtw + k);
        const R cx = w.x * b.x + w.y * b.y, cy = w.x * b.y - w.y * b.x;
        z = mkc(a.x - cy, a.y + cx);
      }
      A[l * g.ls + k] = z;
    }
    __syncthreads();
    prefetch(e + 1);   // the staging buffer has been read: the next entry's copy runs under this one's stages
    fft_lines<R, true>(A, B, nl, g.ls, fnl, plan);
    return true;
  };

  int e = 0;   // the next entry (after a failed wait: the entry that failed)
  bool ok = true;
  while (ok && e < e_lo + e_k0) {
    ok = c2r_entry(e);
    if (ok) ++e;
  }
  for (int k = k0; ok && k < k1; ++k) {
    if (needs_next(k)) {
      ok = c2r_entry(e);
      if (!ok) break;
      ++e;
    }
    const long long orow = ((long long)inst * g.nz + (k - 1)) * g.ny2;
    if (k > g.nz - 1) {
      // no product at the lid level
      for (int t = threadIdx.x; t < nl3 * g.K; t += blockDim.x) {
        const int l = g.fK.div(t), kk = t - l * g.K;
        const int f = g.frt.div(l), r = l - f * rt;
        if (r < rows) out[(long long)f * g.out_fs + (orow + row0 + r) * g.K + kk] = czero<T2>();
      }
      continue;
    }
    // products at level k (the arithmetic of the 3/2-grid loader of the
    // three-pass form, convec.f90:176-200 and :224-243)
    const R* Z0 = slot_z(k);
    const R* Zp = slot_z(k + 1);   // read only where needs_next(k)
    const R* Zm = slot_z(k + 2);   // level k-1 (read only for k >= 2)
    T2* PA = S;
    T2* PB = S + (long long)nl3 * g.ls;
    const int lsr = 2 * g.ls;
    for (int t = threadIdx.x; t < rt * H; t += blockDim.x) {
      const int r = g.fH.div(t), n = t - r * H;
      R cxv[2], cyv[2], czv[2];
#pragma unroll
      for (int e2 = 0; e2 < 2; ++e2) {
        const int i = 2 * n + e2;
        auto at = [&](const R* Z, int f) { return Z[(f * rt + r) * lsr + i]; };
        const R h = FftConst<R>::half();
        const R ub = at(Z0, 0), vb = at(Z0, 1), wb = at(Z0, 2);
        const R o1 = at(Z0, 3), o2 = at(Z0, 4), o3 = at(Z0, 5);
        R cx, cy, cz;
        if (k == 1) {
          const R wbp = at(Zp, 2), o1p = at(Zp, 3), o2p = at(Zp, 4);
          cx = c * (vb * (-o3) + h * wbp * (o2p));
          cy = c * (ub * (o3) + h * wbp * (-o1p));
        } else if (k == g.nz - 1) {
          cx = c * (vb * (-o3) + h * wb * (o2));
          cy = c * (ub * (o3) + h * wb * (-o1));
        } else {
          const R wbp = at(Zp, 2), o1p = at(Zp, 3), o2p = at(Zp, 4);
          cx = c * (vb * (-o3) + h * (wbp * (o2p) + wb * (o2)));
          cy = c * (ub * (o3) + h * (wbp * (-o1p) + wb * (-o1)));
        }
        if (k == 1) {
          cz = FftConst<R>::zero();
        } else {
          const R ubm = at(Zm, 0), vbm = at(Zm, 1);
          cz = c * h * ((ub + ubm) * (-o2) + (vb + vbm) * (o1));
        }
        cxv[e2] = cx; cyv[e2] = cy; czv[e2] = cz;
      }
      PA[(0 * rt + r) * g.ls + n] = mkc(cxv[0], cxv[1]);
      PA[(1 * rt + r) * g.ls + n] = mkc(cyv[0], cyv[1]);
      PA[(2 * rt + r) * g.ls + n] = mkc(czv[0], czv[1]);
    }
    __syncthreads();
    const T2* Z = fft_lines<R, false>(PA, PB, nl3, g.ls, g.f3, plan);
    for (int t = threadIdx.x; t < nl3 * g.K; t += blockDim.x) {
      const int l = g.fK.div(t), kk = t - l * g.K;
      const int f = g.frt.div(l), r = l - f * rt;
      if (r >= rows) continue;
      const T2 zk = Z[l * g.ls + kk];
      const T2 zm = Z[l * g.ls + (kk == 0 ? 0 : H - kk)];
      const T2 a = cadd_conj(zk, zm);
      const T2 b = csub_conj(zk, zm);
      const T2 w = ldt(plan.rtw + kk);
      const R wbx = w.x * b.x - w.y * b.y, wby = w.x * b.y + w.y * b.x;
      out[(long long)f * g.out_fs + (orow + row0 + r) * g.K + kk] = mkc(rmul_half(a.x + wby), rmul_half(a.y - wbx));
    }
    __syncthreads();
  }
  if (!ok) {
    // a copy wait gave up: record it, give the copies of that entry (the
    // only ones in flight; the next were not issued) a last bounded wait,
    // and leave
    if (threadIdx.x == 0) atomicExch(g.err, 1);
    mbar_wait(bar, (unsigned)(e & 1));
  }
}

}  // namespace lesgo
