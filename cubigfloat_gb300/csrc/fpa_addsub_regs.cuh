// fpa_addsub_regs.cuh -- add/sub with the operands held in registers, K limbs per lane.
//
// For n <= G*K each lane l of a group holds limbs l*K .. l*K+K-1 of both operands (one
// 16-byte load per operand per lane when K = 4), so an add/sub reads its operands once
// from HBM, never touches shared memory and writes its result once.  Word shifts by a
// group-uniform amount are a rotation of the K slots plus K+1 shuffles; carries and
// borrows between lanes are resolved by a ballot lookahead.
//
// The result is the same as op_addsub_staged's: the aligned sum
//   X = BIG * 2^64 +- floor(SMALL * 2^(64-d))
// is formed exactly in n+3 limbs (X limbs 0 and 1 are the guard limbs, every lane holds
// K of the limbs 2 .. G*K+1, and X limb G*K+2 is the carry out of an add with n = G*K),
// bits of SMALL below X limb 0 become a sticky flag (and one unit borrowed for an
// effective subtraction), and X is rounded once.  Reference: fpa_warp_add_sub.h:310-380
// (dispatch), :41-125 (same-sign add), :127-282 (effective subtraction); range checks as
// there (:118-119, :226-227, :272-273).
#pragma once
#include <cuda_runtime.h>
#include "fpa_ops.cuh"
#include "fpa_launch.h"

namespace gfpa {

template <int K>
struct Log2 { static constexpr int v = (K <= 1) ? 0 : 1 + Log2<K / 2>::v; };

// v'[i] = v[(i + r) mod K] for a group-uniform r in [0, K)
template <int K>
__device__ __forceinline__ void rotate_slots(uint32_t (&v)[K], int r) {
#pragma unroll
  for (int b = 1; b < K; b <<= 1) {
    const bool f = (r & b) != 0;
    uint32_t t[K];
#pragma unroll
    for (int i = 0; i < K; i++) t[i] = f ? v[(i + b) & (K - 1)] : v[i];
#pragma unroll
    for (int i = 0; i < K; i++) v[i] = t[i];
  }
}

// the group-uniform limb `idx` of a group vector (0 outside [0, G*K))
template <int G, int K>
__device__ __forceinline__ uint32_t limb_at(const Grp<G> &g, const uint32_t (&v)[K], int idx) {
  const int slot = idx & (K - 1), lane = idx >> Log2<K>::v;
  uint32_t s = v[0];
#pragma unroll
  for (int i = 1; i < K; i++) s = slot == i ? v[i] : s;
  const uint32_t r = __shfl_sync(g.mask, s, lane & (G - 1), G);
  return (idx >= 0 && idx < G * K) ? r : 0u;
}

// out[t] = limb (l*K + off + t) of the group vector v for t = 0..K; limbs outside [0, G*K)
// read as 0.  `off` is group-uniform and may be negative.
template <int G, int K>
__device__ __forceinline__ void window(const Grp<G> &g, const uint32_t (&v)[K], int off, uint32_t (&out)[K + 1]) {
  const int q = off >> Log2<K>::v, r = off & (K - 1);   // floor division, also for off < 0
  uint32_t rot[K];
#pragma unroll
  for (int i = 0; i < K; i++) rot[i] = v[i];
  rotate_slots<K>(rot, r);
#pragma unroll
  for (int t = 0; t <= K; t++) {
    const int src = (int)g.lane + q + ((r + t) >= K ? 1 : 0);
    const uint32_t val = __shfl_sync(g.mask, rot[t & (K - 1)], src & (G - 1), G);
    out[t] = ((unsigned)src < (unsigned)G) ? val : 0u;
  }
}

// K limbs of lane l from a[l*K ..], zero at and above n
template <int G, int K>
__device__ __forceinline__ void load_slots(const Grp<G> &g, const uint32_t *a, int n, bool vec, uint32_t (&v)[K]) {
  const int base = (int)g.lane * K;
  if constexpr (K % 4 == 0) {
    if (vec && base + K <= n) {
#pragma unroll
      for (int j = 0; j < K / 4; j++) {
        const uint4 w = __ldcs(reinterpret_cast<const uint4 *>(a + base) + j);
        v[4 * j] = w.x; v[4 * j + 1] = w.y; v[4 * j + 2] = w.z; v[4 * j + 3] = w.w;
      }
      return;
    }
  }
  if constexpr (K % 2 == 0) {
    if (vec && base + K <= n) {
#pragma unroll
      for (int j = 0; j < K / 2; j++) {
        const uint2 w = __ldcs(reinterpret_cast<const uint2 *>(a + base) + j);
        v[2 * j] = w.x; v[2 * j + 1] = w.y;
      }
      return;
    }
  }
#pragma unroll
  for (int s = 0; s < K; s++) v[s] = base + s < n ? __ldcs(a + base + s) : 0u;
}

template <int G, int K>
__device__ __forceinline__ void store_slots(const Grp<G> &g, uint32_t *r, int n, bool vec, const uint32_t (&v)[K]) {
  const int base = (int)g.lane * K;
  if constexpr (K % 4 == 0) {
    if (vec && base + K <= n) {
#pragma unroll
      for (int j = 0; j < K / 4; j++)
        __stcs(reinterpret_cast<uint4 *>(r + base) + j, make_uint4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]));
      return;
    }
  }
  if constexpr (K % 2 == 0) {
    if (vec && base + K <= n) {
#pragma unroll
      for (int j = 0; j < K / 2; j++) __stcs(reinterpret_cast<uint2 *>(r + base) + j, make_uint2(v[2 * j], v[2 * j + 1]));
      return;
    }
  }
#pragma unroll
  for (int s = 0; s < K; s++)
    if (base + s < n) __stcs(r + base + s, v[s]);
}

// One add/sub of two operands held in registers (n <= G*K; slots at and above n are 0).
// `vec` allows vector stores to r (r 16-byte aligned and n a multiple of 4).
// An effective subtraction is the addition of the ones' complement of the aligned SMALL
// with a carry in of 1 - lost (X = BIG*2^64 + ~T + 1 - lost mod 2^(32(G*K+2))), so add and
// sub share one code path; the common alignments of the result (no cancellation, or one
// limb of it) are handled without branches.
template <int G, int K>
__device__ __forceinline__ void op_addsub_regk(const Grp<G> &g, int n, int mode, int is_sub, bool vec,
                                               uint32_t a_exp, const uint32_t (&av)[K], uint32_t b_exp,
                                               const uint32_t (&bv)[K], uint32_t *r_exp, uint32_t *r) {
  static_assert(K >= 2 && (K & (K - 1)) == 0, "K is a power of two >= 2");
  constexpr int GK = G * K;
  const int l = (int)g.lane, base = l * K;
  const uint32_t act = c_action[is_sub][classify(a_exp) * 9 + classify(b_exp)];
  if (act == ACT_COPY_A) {
    store_slots<G, K>(g, r, n, vec, av);
    if (l == 0) *r_exp = a_exp;
    return;
  }
  if (act == ACT_COPY_B || act == ACT_NEG_B) {                 // b, or 0 - b = -b
    store_slots<G, K>(g, r, n, vec, bv);
    if (l == 0) *r_exp = act == ACT_COPY_B ? b_exp : (b_exp ^ 1u);
    return;
  }
  if (act != ACT_ADD && act != ACT_SUB) { if (l == 0) *r_exp = act; return; }
  const uint32_t sa = a_exp & 1u, sb = (b_exp & 1u) ^ (uint32_t)is_sub;
  const uint32_t wa = a_exp >> 1, wb = b_exp >> 1;             // BIAS + e
  const bool eff_sub = sa != sb;
  bool a_big;
  if (wa != wb) a_big = wa > wb;
  else {                                                       // compare the mantissas
    int ts = -1;
#pragma unroll
    for (int s = 0; s < K; s++) if (av[s] != bv[s]) ts = s;
    const uint32_t dm = g.ballot(ts >= 0);
    uint32_t gt = 0;
#pragma unroll
    for (int s = 0; s < K; s++) if (s == ts) gt = av[s] > bv[s] ? 1u : 0u;
    const uint32_t top_gt = g.bcast(gt, dm ? 31 - __clz((int)dm) : 0);
    if (dm == 0 && eff_sub) { if (l == 0) *r_exp = CLS_ZERO; return; }   // exact cancellation
    a_big = dm == 0 || top_gt != 0;
  }
  uint32_t big[K], sml[K];
#pragma unroll
  for (int s = 0; s < K; s++) { big[s] = a_big ? av[s] : bv[s]; sml[s] = a_big ? bv[s] : av[s]; }
  const uint32_t sign = a_big ? sa : sb;
  const uint32_t wbig = a_big ? wa : wb, diff = a_big ? wa - wb : wb - wa;
  const uint32_t cap = 32u * (uint32_t)n + 64u;
  const int d = (int)(diff > cap ? cap : diff);
  const int dw = d >> 5, db = d & 31;

  // T = floor(SMALL * 2^(64-d)): every lane's limbs 2+base .. 2+base+K-1 come from SMALL
  // limbs base+dw .. base+dw+K; the guard limbs T[0], T[1] from SMALL limbs dw-2 .. dw.
  uint32_t sh[K], t0, t1;
  {
    const int q = dw >> Log2<K>::v, rr = dw & (K - 1);
    uint32_t rot[K];
#pragma unroll
    for (int i = 0; i < K; i++) rot[i] = sml[i];
    rotate_slots<K>(rot, rr);
    uint32_t w[K + 1];
#pragma unroll
    for (int t = 0; t <= K; t++) {
      const int src = l + q + ((rr + t) >= K ? 1 : 0);
      const uint32_t val = __shfl_sync(g.mask, rot[t & (K - 1)], src & (G - 1), G);
      w[t] = src < G ? val : 0u;
    }
#pragma unroll
    for (int s = 0; s < K; s++) sh[s] = __funnelshift_r(w[s], w[s + 1], db);
    const int l1 = q - (rr < 1 ? 1 : 0), l2 = q - (rr < 2 ? 1 : 0);
    const uint32_t v1 = __shfl_sync(g.mask, rot[K - 1], l1 & (G - 1), G);
    const uint32_t v2 = __shfl_sync(g.mask, rot[K - 2], l2 & (G - 1), G);
    const uint32_t sm1 = (unsigned)l1 < (unsigned)G ? v1 : 0u;           // SMALL[dw-1]
    const uint32_t sm2 = (unsigned)l2 < (unsigned)G ? v2 : 0u;           // SMALL[dw-2]
    const uint32_t s0v = g.bcast(w[0], 0);                                // SMALL[dw]
    t0 = __funnelshift_r(sm2, sm1, db);
    t1 = __funnelshift_r(sm1, s0v, db);
  }
  // bits of SMALL below T[0] (d > 64): sticky, and one unit less for an effective subtraction
  uint32_t lost;
  {
    const int cut = d - 64, full = cut >> 5, part = cut & 31;  // nothing is lost for cut <= 0
    uint32_t lv = 0;
#pragma unroll
    for (int s = 0; s < K; s++) {
      const int idx = base + s;
      lv |= sml[s] & (idx < full ? 0xFFFFFFFFu : (idx == full ? ((1u << part) - 1u) : 0u));
    }
    lost = g.ballot(lv != 0) != 0 ? 1u : 0u;
  }
  // X = BIG*2^64 + (T ^ msk) + cin0:  X[0], X[1] in every lane, X[2 + base + s] in x[s]
  const uint32_t msk = eff_sub ? 0xFFFFFFFFu : 0u;
  uint32_t x0, x1, cin;
  {
    const uint64_t u0 = (uint64_t)(t0 ^ msk) + (eff_sub ? 1u - lost : 0u);
    const uint64_t u1 = (uint64_t)(t1 ^ msk) + (uint32_t)(u0 >> 32);
    x0 = (uint32_t)u0; x1 = (uint32_t)u1; cin = (uint32_t)(u1 >> 32);
  }
  uint32_t x[K];
  {
    uint32_t c = 0, all1 = 0xFFFFFFFFu;
#pragma unroll
    for (int s = 0; s < K; s++) {
      const uint64_t u = (uint64_t)big[s] + (sh[s] ^ msk) + c;
      x[s] = (uint32_t)u; c = (uint32_t)(u >> 32); all1 &= x[s];
    }
    uint32_t cout;
    const uint64_t cv = lookahead<G>(g.ballot(c != 0), g.ballot(all1 == 0xFFFFFFFFu && c == 0), cin, cout);
    uint32_t ci = (uint32_t)(cv >> l) & 1u;
#pragma unroll
    for (int s = 0; s < K; s++) { const uint64_t u = (uint64_t)x[s] + ci; x[s] = (uint32_t)u; ci = (uint32_t)(u >> 32); }
    cin = eff_sub ? 0u : cout;                                 // X limb G*K+2 (only when n == G*K)
  }
  const uint32_t xtop = cin;

  // bit length of X
  int L;
  {
    int ts = -1; uint32_t tv = 0;
#pragma unroll
    for (int s = 0; s < K; s++) if (x[s]) { ts = s; tv = x[s]; }
    const uint32_t nz = g.ballot(ts >= 0);
    const int myL = 32 * (base + ts + 2) + 32 - (int)clz32(tv);
    const int topL = g.bcast((uint32_t)myL, nz ? 31 - __clz((int)nz) : 0);
    if (xtop) L = 32 * (GK + 2) + 32 - (int)clz32(xtop);
    else if (nz) L = topL;
    else if (x1) L = 64 - (int)clz32(x1);
    else if (x0) L = 32 - (int)clz32(x0);
    else { if (l == 0) *r_exp = CLS_ZERO; return; }
  }
  const int lo = L - 32 * n;                                   // bit of X at the mantissa's bit 0
  const int lw = lo >> 5, lb = lo & 31;                        // floor division
  const int off = lw - 2;                                      // mantissa limb i = X[i+lw..] = x[i+off..]
  uint32_t m[K + 1], rbit = 0, st = 0;
  const uint32_t nx = __shfl_down_sync(g.mask, x[0], 1, G);
  const uint32_t pv = __shfl_up_sync(g.mask, x[K - 1], 1, G);
  if (off == 0 || off == -1) {                                 // no cancellation, or one limb
    const bool f0 = off == 0;
    m[0] = f0 ? x[0] : (l == 0 ? x1 : pv);
#pragma unroll
    for (int t = 1; t < K; t++) m[t] = f0 ? x[t] : x[t - 1];
    m[K] = f0 ? (l == G - 1 ? xtop : nx) : x[K - 1];
    // the round bit lies in X limb 0, 1 or 2 (lo in [32, 96))
    const int rp = lo - 1, rk = rp >> 5, rq = rp & 31;
    const uint32_t x2 = g.bcast(x[0], 0);
    const uint32_t xr = rk == 0 ? x0 : (rk == 1 ? x1 : x2);
    rbit = (xr >> rq) & 1u;
    st = ((rk > 0 ? x0 : 0u) | (rk > 1 ? x1 : 0u) | (xr & ((1u << rq) - 1u))) != 0u ? 1u : 0u;
  } else {                                                     // deep cancellation (exact result)
    window<G, K>(g, x, off, m);
#pragma unroll
    for (int t = 0; t <= K; t++) {
      const int mi = base + off + t;
      if (mi == -1) m[t] = x1;
      else if (mi == -2) m[t] = x0;
      else if (mi == GK) m[t] = xtop;
    }
    if (lo >= 1) {
      const int rp = lo - 1, rk = rp >> 5;
      const uint32_t xm = limb_at<G, K>(g, x, rk - 2);
      const uint32_t xr = rk == 0 ? x0 : (rk == 1 ? x1 : (rk == GK + 2 ? xtop : xm));
      rbit = (xr >> (rp & 31)) & 1u;
      uint32_t part = 0;
#pragma unroll
      for (int s = 0; s < K; s++) if (base + s + 2 < rk) part |= x[s];
      if (l == 0) {
        if (rk > 0) part |= x0;
        if (rk > 1) part |= x1;
        if (rp & 31) part |= xr & ((1u << (rp & 31)) - 1u);
      }
      st = g.ballot(part != 0) != 0 ? 1u : 0u;
    }
  }
  uint32_t mant[K];
#pragma unroll
  for (int s = 0; s < K; s++) mant[s] = base + s < n ? __funnelshift_r(m[s], m[s + 1], lb) : 0u;

  // round: add one unit with carry lookahead (every lane whose lower lanes are all ones)
  const uint32_t lsb = g.bcast(mant[0], 0) & 1u;
  const bool up = round_up(mode, sign, lsb, rbit, st | lost);
  bool ones = true;
#pragma unroll
  for (int s = 0; s < K; s++) ones = ones && (base + s >= n || mant[s] == 0xFFFFFFFFu);
  const uint32_t om = g.ballot(ones);
  const uint32_t below = (1u << l) - 1u;                       // l < 32
  uint32_t ci = (up && (om & below) == below) ? 1u : 0u;
#pragma unroll
  for (int s = 0; s < K; s++) {
    const uint32_t v = mant[s] + ci;
    ci = (ci && v == 0u) ? 1u : 0u;
    mant[s] = base + s < n ? v : 0u;
  }
  const uint32_t need = (G == 32) ? 0xFFFFFFFFu : ((1u << G) - 1u);
  const int ovf = (up && (om & need) == need) ? 1 : 0;         // 0.11..1 + ulp = 1.0
#pragma unroll
  for (int s = 0; s < K; s++) mant[s] = ovf ? ((base + s == n - 1) ? 0x80000000u : 0u) : mant[s];
  const long long be = (long long)wbig - 32LL * n - 64 + L + ovf;   // BIAS + e
  if (!eff_sub && be > 0x7FFFFFFFLL) { if (l == 0) *r_exp = CLS_POS_INF - sign; return; }
  if (eff_sub && be < 5) { if (l == 0) *r_exp = CLS_POS_TINY - sign; return; }
  store_slots<G, K>(g, r, n, vec, mant);
  if (l == 0) *r_exp = (uint32_t)(2 * be) + sign;
}

// add/sub of numbers that fit K limbs per lane (n <= G*K): registers and shuffles only.
// Each group loads the next operation's operands while it computes the current one.
template <int OP, int G, int K>
__global__ void __launch_bounds__(128, (K <= 4) ? 8 : (K <= 8 ? 4 : 2)) k_addsub_regk(ElementwiseArgs args) {
  Grp<G> g;
  const uint32_t gpc = blockDim.x / G, gi = threadIdx.x / G;
  const int n = (int)args.n;
  const bool vec = (n & 3) == 0 &&
                   ((((uintptr_t)args.a_limbs) | ((uintptr_t)args.b_limbs) | ((uintptr_t)args.r_limbs)) & 15) == 0;
  const uint64_t stride = (uint64_t)gridDim.x * gpc;
  uint64_t i = (uint64_t)blockIdx.x * gpc + gi;
  uint32_t av[K], bv[K], ae = 0, be = 0;
  if (i < args.count) {
    load_slots<G, K>(g, args.a_limbs + i * n, n, vec, av);
    load_slots<G, K>(g, args.b_limbs + i * n, n, vec, bv);
    ae = args.a_exps[i]; be = args.b_exps[i];
  }
  for (; i < args.count; i += stride) {
    const uint64_t nx = i + stride;
    uint32_t nav[K], nbv[K], nae = 0, nbe = 0;
#pragma unroll
    for (int s = 0; s < K; s++) { nav[s] = 0u; nbv[s] = 0u; }
    if (nx < args.count) {
      load_slots<G, K>(g, args.a_limbs + nx * n, n, vec, nav);
      load_slots<G, K>(g, args.b_limbs + nx * n, n, vec, nbv);
      nae = args.a_exps[nx]; nbe = args.b_exps[nx];
    }
    op_addsub_regk<G, K>(g, n, args.mode, OP == OP_SUB, vec, ae, av, be, bv, args.r_exps + i,
                         args.r_limbs + i * (uint64_t)n);
#pragma unroll
    for (int s = 0; s < K; s++) { av[s] = nav[s]; bv[s] = nbv[s]; }
    ae = nae; be = nbe;
  }
}

template <int OP, int G, int K>
static cudaError_t launch_addsub_regk(const ElementwiseArgs &args, cudaStream_t stream, int sms) {
  static int per_sm = 0;
  auto kern = k_addsub_regk<OP, G, K>;
  if (per_sm == 0) {
    int b = 0;
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, 128, 0);
    if (e != cudaSuccess) return e;
    per_sm = b < 1 ? 1 : b;
  }
  constexpr int gpc = 128 / G;
  const uint64_t need = (args.count + gpc - 1) / gpc, cap = (uint64_t)sms * per_sm;
  const unsigned grid = (unsigned)(need < cap ? need : cap);
  if (grid == 0) return cudaSuccess;
  kern<<<grid, 128, 0, stream>>>(args);
  return cudaGetLastError();
}

}  // namespace gfpa
