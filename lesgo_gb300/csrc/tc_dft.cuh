// The x-direction real-to-complex transform as a tensor-core GEMM: each row
// of M reals (x) times the M x M real DFT matrix W gives the row's M/2 kept
// modes (re, im interleaved), the same values k_xfwd computes with the
// radix stages (fft.f90:114-121 forward r2c, FFTW's unnormalised sign
// convention; the Nyquist mode is not kept).
//
// Tensor cores (tcgen05.mma kind::tf32, accumulators in tensor memory).  TF32
// keeps 10 mantissa bits, so every operand is split into hi = x with the low
// 13 mantissa bits cleared (exact in TF32) and lo = x - hi (exact in FP32),
// and the product is hi*Whi + (hi*Wlo + lo*Whi): the dropped lo*Wlo term and
// lo's own rounding are below 2^-21 of each product.  The large term and the
// two small ones accumulate in separate tensor-memory accumulators (the
// tensor cores' FP32 accumulation rounds at every 8-term step, so the large
// term's accumulator sees M/8 roundings instead of 3M/8) and the epilogue
// adds them.
//
// Work: a tile is 128 GEMM rows (rpc rows of each of NF fields, m = f*rpc+r;
// spare rows are zero); persistent blocks walk the tiles, each tile in
// chunks of 16 x values.  Warp roles:
//   warps 0-7   producers, two teams of four warps taking alternate groups
//               of chunks: load a group's values through Src (several
//               chunks at once, so that many loads are in flight), split
//               them and store them into a ring of kXdStages stage buffers;
//   warps 8-11  epilogue: read a finished tile's accumulators (tcgen05.ld,
//               warp w reads lanes 32*(w-8)..), add them, store the modes;
//   warp 12     allocates tensor memory; its lane 0 waits for W (copied once
//               per block by a bulk copy) and issues the MMAs of each chunk.
// Barriers: full[s] (the 4 warps of the chunk's team arrive), empty[s] (tcgen05.commit
// once the chunk's MMAs have read it), acc_full[a] (commit at a tile's last
// chunk), acc_empty[a] (the 4 epilogue warps arrive); two accumulator sets
// let the MMAs of tile t+1 run while the epilogue drains tile t.  Every
// wait is bounded; a wait that runs out sets an abort flag that ends every
// role's loop, and the device error flag.
//
// Shared-memory operand layout: K-major, no swizzle.  A core matrix is 8
// rows x 16 bytes (8 x 4 TF32 values), stored contiguously.  Element (m, k)
// of a staged chunk sits at (m/8)*kSboA + (k/4)*kLboA + (m%8)*16 + (k%4)*4
// bytes; the leading offset (between the 4 core matrices along K) is 192
// bytes so that a warp's stores (4 rows x 8 pairs) fall on every bank
// twice, the minimum for 8-byte stores.  W is [n][x] with a leading offset
// of 128 and a stride offset of M/4 * 128.
#pragma once
#include "bulk_copy.cuh"
#include "fft_core.cuh"

#include <cmath>
#include <cstring>
#include <vector>

namespace lesgo {

constexpr int kXdKc = 16;                      // x values per staged chunk
constexpr unsigned kLboA = 192;                // bytes between core matrices along K
constexpr unsigned kSboA = 4 * kLboA;          // bytes between 8-row groups
constexpr unsigned kXdPiece = 16 * kSboA;      // one staged piece (hi or lo) of a chunk
constexpr int kXdStages = 4;
static_assert(kXdStages % 4 == 0, "two teams in groups of kXdStages / 2 chunks");
constexpr int kXdProducers = 256;              // warps 0-7
constexpr int kXdTeam = 128;                   // producer warps per team (two teams)
constexpr int kXdThreads = 13 * 32;            // + 4 epilogue warps + the MMA warp

struct XdGeom {
  int M;          // real row length (nx): a multiple of 16, at most 128
  int K;          // modes kept (M/2); a row's output is 2K = M reals
  int nrows;      // rows per field in this launch
  int nyrows;     // rows per level
  int rpc;        // rows of each field per tile (NF * rpc <= 128)
  int ntiles;
  unsigned ncols;              // tensor-memory columns allocated
  unsigned pcols;              // columns per accumulator (M rounded up to 32)
  long long out_field_stride;  // complex elements between fields in the output
  FastDiv fnyrows;             // by nyrows
  int* err;                    // set when a wait runs out
};

// ---- tcgen05 / tensor-memory primitives -----------------------------------
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// warp-collective: the allocated column base is written to *slot
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, unsigned ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, unsigned ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// shared-memory matrix descriptor: no swizzle, descriptor version 1
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46);
}
// instruction descriptor, kind::tf32: D FP32, A and B TF32, both K-major, M = 128
__host__ __device__ constexpr uint32_t idesc_tf32(int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
// arrives on `bar` once every MMA this thread issued before has completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}
// warp-collective: 16 consecutive 32-bit columns of the warp's 32 lanes (lane
// = the thread's lane within the warp's quarter), waited for in place
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
}

__device__ __forceinline__ float tf32_hi(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }


// polls like mbar_wait, and gives up early once another thread has aborted
__device__ __forceinline__ bool mbar_wait_abort(uint64_t* bar, unsigned parity, volatile int* abort) {
  const unsigned a = smem_addr(bar);
  for (unsigned it = 0; it < kMbarPollLimit; ++it) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (*abort) return false;
  }
  return false;
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Dynamic shared memory of k_xdft_tc: W (hi, lo), the stage ring (hi and lo
// pieces), the barriers, the tensor-memory slot and the abort flag.
__host__ __device__ inline size_t xdft_smem(int M) {
  return 2ull * M * M * 4 + 2ull * kXdStages * kXdPiece + 8 * (2 * kXdStages + 5) + 16;
}

// (row, x pair) items a producer thread holds per chunk, and chunks loaded
// at once (registers: chunks x items x NF complex values)
__host__ __device__ constexpr int xd_ipc(int nf) { return (128 / nf * (kXdKc / 2) + kXdTeam - 1) / kXdTeam; }
// A team's groups are G consecutive chunks and the teams alternate, so ring
// slot s (chunk q at q % kXdStages) belongs to one team as long as
// kXdStages / G is even: every wait on a slot's empty barrier is then for the
// phase right after the one its own team last waited for (a wait two phases
// ahead would pass on the earlier phase's parity).
__host__ __device__ constexpr int xd_group(int nf) { return nf > 6 ? 1 : kXdStages / 2; }

template <int NF, class Src>
__global__ void __launch_bounds__(kXdThreads, 1)
    k_xdft_tc(XdGeom g, const float* __restrict__ wimg, Src src, float2* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int IPC = xd_ipc(NF), G = xd_group(NF), S = kXdStages;
  const int M = g.M;
  const unsigned wbytes = (unsigned)M * M * 4, sboB = (unsigned)(M / 4) * 128;
  unsigned char* Wh = smem_raw;
  unsigned char* Wl = smem_raw + wbytes;
  unsigned char* ring = smem_raw + 2 * wbytes;                 // stage s: hi at 2s, lo at 2s+1
  uint64_t* full = reinterpret_cast<uint64_t*>(ring + 2 * S * kXdPiece);
  uint64_t* empty = full + S;
  uint64_t* accf = empty + S;
  uint64_t* acce = accf + 2;
  uint64_t* wbar = acce + 2;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(wbar + 1);
  volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nch = M / kXdKc;
  const int my_tiles = blockIdx.x < g.ntiles ? (g.ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int nq = my_tiles * nch;   // chunks of this block

  // zero the ring once: rows m >= NF*rpc stay zero
  for (unsigned i = tid * 16; i < 2 * S * kXdPiece; i += kXdThreads * 16)
    *reinterpret_cast<uint4*>(ring + i) = make_uint4(0, 0, 0, 0);
  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], kXdTeam / 32);
      mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(&accf[a], 1);
      mbar_init(&acce[a], 4);
    }
    mbar_init(wbar, 1);
    *abort = 0;
    mbar_init_fence();
  }
  if (warp == 12) tmem_alloc(tslot, g.ncols);
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp < 8) {
    // ---------------- producers ----------------
    // two teams of four warps take alternate groups of G chunks: one team's
    // loads are in flight while the other stores its group into the ring
    const int team = warp >> 2, ttid = tid & (kXdTeam - 1);
    for (int q0 = team * G; q0 < nq && !*abort; q0 += 2 * G) {
      float2 v[G][IPC][NF];
#pragma unroll
      for (int j = 0; j < G; ++j) {
        const int q = q0 + j;
        const int tile = blockIdx.x + (q / nch) * gridDim.x, c = q % nch;
        const int row0 = tile * g.rpc;
#pragma unroll
        for (int i = 0; i < IPC; ++i) {
          const int t = ttid + i * kXdTeam;
          const int r = t >> 3, p = t & 7;
          const int row = row0 + r;
          if (q < nq && r < g.rpc && row < g.nrows) {
            const int li = g.fnyrows.div(row), jy = row - li * g.nyrows;
            typename Src::C w[NF];
            src.load2(c * (kXdKc / 2) + p, jy, li, w);
#pragma unroll
            for (int f = 0; f < NF; ++f) v[j][i][f] = cvt2<float2>(w[f]);
          } else {
#pragma unroll
            for (int f = 0; f < NF; ++f) v[j][i][f] = make_float2(0.f, 0.f);
          }
        }
      }
#pragma unroll
      for (int j = 0; j < G; ++j) {
        const int q = q0 + j;
        if (q >= nq) break;
        const int s = q % S;
        // warp-uniform: every lane of the warp takes the same branch
        if (q >= S && !__all_sync(0xffffffffu, mbar_wait_abort(&empty[s], ((q / S) - 1) & 1, abort))) {
          *abort = 1;
          break;
        }
        unsigned char* Ah = ring + (2 * s) * kXdPiece;
        unsigned char* Al = Ah + kXdPiece;
#pragma unroll
        for (int i = 0; i < IPC; ++i) {
          const int t = ttid + i * kXdTeam;
          const int r = t >> 3, k = 2 * (t & 7);
          if (r < g.rpc) {
#pragma unroll
            for (int f = 0; f < NF; ++f) {
              const int m = f * g.rpc + r;
              const unsigned off = (unsigned)(m >> 3) * kSboA + (unsigned)(k >> 2) * kLboA + (m & 7) * 16 + (k & 3) * 4;
              const float hx = tf32_hi(v[j][i][f].x), hy = tf32_hi(v[j][i][f].y);
              *reinterpret_cast<float2*>(Ah + off) = make_float2(hx, hy);
              *reinterpret_cast<float2*>(Al + off) =
                  make_float2(__fsub_rn(v[j][i][f].x, hx), __fsub_rn(v[j][i][f].y, hy));
            }
          }
        }
        fence_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&full[s]);
      }
    }
  } else if (warp < 12) {
    // ---------------- epilogue ----------------
    const int quarter = warp - 8;
    const int m = quarter * 32 + lane;
    const int f = m / g.rpc, r = m - f * g.rpc;
    for (int k = 0; k < my_tiles; ++k) {
      const int a = k & 1;
      if (!__all_sync(0xffffffffu, mbar_wait_abort(&accf[a], (k >> 1) & 1, abort))) {
        *abort = 1;
        break;
      }
      tc_fence_after();
      const int tile = blockIdx.x + k * gridDim.x;
      const int row = tile * g.rpc + r;
      const bool live = f < NF && row < g.nrows;
      float2* dst = out + (live ? (long long)f * g.out_field_stride + (long long)row * g.K : 0);
      const uint32_t base = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(a * 2 * g.pcols);
      for (int cc = 0; cc < M / 16; ++cc) {
        uint32_t big[16], sml[16];
        tmem_ld16(base + (uint32_t)(cc * 16), big);
        tmem_ld16(base + g.pcols + (uint32_t)(cc * 16), sml);
        if (live) {
          float4* d4 = reinterpret_cast<float4*>(dst + cc * 8);
#pragma unroll
          for (int j = 0; j < 4; ++j)
            d4[j] = make_float4(__uint_as_float(big[4 * j]) + __uint_as_float(sml[4 * j]),
                                __uint_as_float(big[4 * j + 1]) + __uint_as_float(sml[4 * j + 1]),
                                __uint_as_float(big[4 * j + 2]) + __uint_as_float(sml[4 * j + 2]),
                                __uint_as_float(big[4 * j + 3]) + __uint_as_float(sml[4 * j + 3]));
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[a]);
    }
  } else if (lane == 0) {
    // ---------------- MMA issue ----------------
    const uint32_t idesc = idesc_tf32(M);
    bool ok = true;
    if (wimg) {
      mbar_arrive_expect_tx(wbar, 2 * wbytes);
      bulk_g2s(Wh, wimg, wbytes, wbar);
      bulk_g2s(Wl, wimg + (size_t)M * M, wbytes, wbar);
      ok = mbar_wait_abort(wbar, 0, abort);
    }
    const uint32_t wh0 = smem_addr(Wh), wl0 = smem_addr(Wl);
    int q = 0;
    for (int k = 0; k < my_tiles && ok; ++k) {
      const int a = k & 1;
      if (k >= 2 && !mbar_wait_abort(&acce[a], ((k >> 1) - 1) & 1, abort)) { ok = false; break; }
      const uint32_t dbig = tmem + (uint32_t)(a * 2 * g.pcols), dsml = dbig + g.pcols;
      for (int c = 0; c < nch; ++c, ++q) {
        const int s = q % S;
        if (!mbar_wait_abort(&full[s], (q / S) & 1, abort)) { ok = false; break; }
        tc_fence_after();
        const uint32_t ah0 = smem_addr(ring + (2 * s) * kXdPiece), al0 = ah0 + kXdPiece;
#pragma unroll
        for (int ks = 0; ks < kXdKc / 8; ++ks) {
          const uint32_t aoff = (uint32_t)ks * 2 * kLboA;
          const uint32_t boff = (uint32_t)((c * kXdKc + ks * 8) >> 2) * 128;
          const uint64_t dah = smem_desc(ah0 + aoff, kLboA, kSboA), dal = smem_desc(al0 + aoff, kLboA, kSboA);
          const uint64_t dbh = smem_desc(wh0 + boff, 128, sboB), dbl = smem_desc(wl0 + boff, 128, sboB);
          const uint32_t first = (c == 0 && ks == 0) ? 0u : 1u;
          mma_tf32(dbig, dah, dbh, idesc, first);
          mma_tf32(dsml, dah, dbl, idesc, first);
          mma_tf32(dsml, dal, dbh, idesc, 1u);
        }
        mma_commit(&empty[s]);
        if (c == nch - 1) mma_commit(&accf[a]);
      }
      if (!ok) break;
    }
    if (!ok) *abort = 1;
    // the MMAs already issued finish before the block's memory is released
    if (q > 0) mbar_wait(&empty[(q - 1) % S], ((q - 1) / S) & 1);
    if (wimg) mbar_wait(wbar, 0);
  }
  __syncthreads();
  if (*abort && tid == 0) atomicExch(g.err, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 12) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tmem, g.ncols);
  }
}

// Host: the W images [hi][lo] of the M x M DFT matrix in the operand layout
// (n = output real: 2k the cosine row, 2k+1 the negative sine row of mode k;
// x = input point).  Angles are reduced exactly ((k x) mod M) and evaluated
// in long double; hi is the TF32 truncation of the FP32 value, lo the
// remainder rounded to FP32.
inline std::vector<float> xdft_image(int M) {
  std::vector<float> img(2 * (size_t)M * M);
  const long double two_pi = 6.283185307179586476925286766559005768L;
  const int sbo = (M / 4) * 32;   // floats between 8-row groups (a core matrix is 32 floats)
  for (int n = 0; n < M; ++n)
    for (int x = 0; x < M; ++x) {
      const long double ang = two_pi * (long double)(((long long)(n / 2) * x) % M) / (long double)M;
      const long double w = (n & 1) ? -std::sin(ang) : std::cos(ang);
      const float wf = (float)w;
      uint32_t u;
      std::memcpy(&u, &wf, 4);
      u &= 0xFFFFE000u;
      float hi;
      std::memcpy(&hi, &u, 4);
      const size_t idx = (size_t)(n / 8) * sbo + (size_t)(x / 4) * 32 + (n % 8) * 4 + (x % 4);
      img[idx] = hi;
      img[(size_t)M * M + idx] = (float)(w - (long double)hi);
    }
  return img;
}

}  // namespace lesgo
