// sr_fit.cu -- fused batched L-BFGS fit of the learnable constants.
//
// One persistent kernel.  Each CTA takes one problem (one tape, one target row)
// from a work queue and runs the complete optimisation for it on chip, its warps
// splitting the N points:
//
//   closure(x)  forward sweep over the tape for the warp's points (lanes over
//               points, operator-node values in shared memory), residuals against
//               Y, then the reverse (adjoint) sweep; the gradient of every constant
//               is summed per lane in float, over the lanes by a butterfly and over
//               the warps in a fixed order, so results are bit-reproducible run to
//               run and the same in every warp.
//   direction   H g over the last `history_size` (s, y) pairs by warp 0, broadcast to
//               the CTA through shared memory: the compact representation (R^-1 and
//               Y^T Y kept up to date as pairs arrive, one lane per pair) for histories
//               of at most 32 pairs, the two-loop recursion for longer ones; scalars as
//               normalised float pairs (Dekker), vectors in float (one slot per lane).
//   line search strong Wolfe (bracket + bisection zoom) or Armijo backtracking, with
//               the reference's acceptance rules and float32 scalar arithmetic.
//
// Per problem the control flow is exactly the reference's LBFGS_batch column
// (symbolic_torch/lbfgs_batch.py:61-326) as driven by optimize()
// (symbolic_torch/optimization.py:51-112).  Every problem of the reference batch
// evolves independently, so the batch-wide early exits of the reference only
// change how much work is done, not the result.  Points the reference evaluates
// twice (phi(0) at the start of each line search and zoom, phi(alpha_lo) at the
// start of a zoom, and the closure after the update when the accepted step was
// already evaluated) are reused here; they are bit-identical because the kernel is
// deterministic.  A problem whose gradient norm drops below tolerance_grad is
// retired at once (the reference keeps computing its unused search direction).
//
// Parameter slots.  The reference optimises all M slots of C but zeroes the
// gradient of every slot that is not a learnable constant; such slots can only
// ever change by picking up NaN through 0*NaN in the vector updates.  Here the
// learnable constants up to the root are the real slots and one extra "virtual"
// slot (gradient always 0) stands for all the others, reproducing that NaN
// propagation through the dots; at the end they are written back as C_init, or as
// NaN when the virtual slot was poisoned.
#include <cstdint>

#include "sr_common.cuh"
#include "sr_ops.cuh"

namespace sr {

__host__ __device__ __forceinline__ size_t fit_align16(size_t x) { return (x + 15) & ~size_t(15); }

struct FitArgs {
  const float* X;
  int64_t N, n_x;
  const float* Y;
  const uint32_t* desc;
  const int32_t* meta;
  int64_t B, M;
  const float* C_init;
  float* C_out;
  int64_t c_sb, c_sm;
  float* Y_final;
  int32_t* iters_out;
  float* loss_out;
  int32_t* evals_out;
  const int32_t* order;
  int max_iter, hist, ls_kind, ls_max, objective;
  double tol, eps;
  int Lmax, Kmax;
  int Imax;         // rows of the per-warp node tables: largest count of operator nodes
  int Amax;         // rows of the per-warp adjoint tables: most operator-node adjoints live at once
  int VR;           // rows of the per-warp table for variables (distinct variables of a tape)
  unsigned char* ws_hist;  // per CTA: the L-BFGS history block (hist_block_bytes), when not in shared memory
  int ring_off;            // > 0: the history block sits in shared memory at this byte offset
  int* counter;
  int32_t* status;
};

// Shared memory.  The CTA works on one problem at a time: the tape, the constants
// published for the current trial point, the slot maps and the cross-warp
// reduction buffers are shared; each warp owns the node table of its own points.
// Float pair of a cascaded sum (Ogita, Rump and Oishi's Sum2): hi is the plain float
// sum of the terms, lo the float sum of the exact rounding errors of those additions
// (Knuth's TwoSum).  hi + lo is as accurate as a sum in twice the precision, rounded
// once; hi alone keeps IEEE semantics (an overflow or an infinite term makes it inf,
// while lo turns NaN), so the total is hi + lo when hi is finite and hi otherwise.
// A pair sum does not depend on the operand order, so a butterfly leaves every lane
// with the same bits.
struct F2 {
  float hi, lo;
};

struct WarpSmem {
  uint32_t* tape;    // [Lmax]                      (CTA)
  uint32_t* pcode;   // [Lmax] opcode of each operator node of the program       (CTA)
  uint32_t* psa;     // [Lmax] operand 0 source word (see the program notes)     (CTA)
  uint32_t* psb;     // [Lmax] operand 1 source word                             (CTA)
  uint32_t* pda;     // [Lmax] operand 0 adjoint destination (byte offset)        (CTA)
  uint32_t* pdb;     // [Lmax] operand 1 adjoint destination                      (CTA)
  int* arow;         // [Lmax] adjoint row of each operator node (by liveness)    (CTA)
  int* frees;        // [Lmax] free adjoint rows while they are assigned          (CTA)
  int* rowvar;       // [VR] variable held in each variable row                  (CTA)
  int* info;         // [8] operator nodes, root row, variable rows, root source, root destination (CTA)
  int* node_slot;    // [Lmax] slot of a LEARNABLE node / row of an operator node / row of a variable (CTA)
  int* slot_node;    // [Kmax]                      (CTA)
  F2* red_g;         // [W][Kmax] per-warp gradient sums (CTA)
  F2* red_l;         // [W] per-warp loss sums      (CTA)
  float* pvec;       // [128] search direction computed by warp 0 (CTA)
  int* red_e;        // [W] per-warp error codes    (CTA)
  long long* task;   // the CTA's current problem   (CTA)
  unsigned char* wb; // this warp's table base (warp):
  float* bc;         //   [1 + Kmax + Lmax] broadcast values: 0, constants, fixed constants
  float* vals;       //   [Imax + VR][32V] operator-node values, then variable values
  float* adj;        //   [Amax + 1][32V] live operator-node adjoints, then a sink row
  float* gl;         //   [Kmax][32V] per-lane, per-point gradient partial sums
};

// Per-warp table layout (byte offsets from the warp's base), V points per lane,
// rows of RW = 32 V floats.
struct WarpLayout {
  uint32_t vals, adj, sink, gl, bytes;
};

__host__ __device__ __forceinline__ WarpLayout warp_layout(int Lmax, int Imax, int Amax, int Kmax, int V, int VR) {
  const uint32_t K = (uint32_t)(Kmax > 0 ? Kmax : 1), I = (uint32_t)(Imax > 0 ? Imax : 1);
  const uint32_t Ar = (uint32_t)(Amax > 0 ? Amax : 1);
  const uint32_t RW = 32u * (uint32_t)V * 4u;  // bytes per row
  WarpLayout w;
  w.vals = (uint32_t)((4u * (1u + K + (uint32_t)Lmax) + 127u) & ~127u);
  w.adj = w.vals + (I + (uint32_t)VR) * RW;
  w.sink = w.adj + Ar * RW;
  w.gl = w.sink + RW;
  w.bytes = w.gl + K * RW;
  return w;
}

__host__ __device__ __forceinline__ size_t fit_shared_bytes(int Lmax, int Kmax, int W, int VR) {
  const size_t K = (size_t)(Kmax > 0 ? Kmax : 1);
  return fit_align16((size_t)Lmax * 4) * 9 + fit_align16(K * 4) + fit_align16((size_t)W * K * 8) +
         fit_align16((size_t)W * 8) + fit_align16((size_t)W * 4) + fit_align16((size_t)VR * 4) + 32 + 16 + 512 +
         128;  // + alignment of the warp tables
}

__host__ __device__ __forceinline__ size_t fit_cta_bytes(int Lmax, int Imax, int Amax, int Kmax, int V, int W,
                                                         int VR) {
  return fit_shared_bytes(Lmax, Kmax, W, VR) + (size_t)W * warp_layout(Lmax, Imax, Amax, Kmax, V, VR).bytes;
}

__device__ __forceinline__ WarpSmem carve(unsigned char* base, int Lmax, int Imax, int Amax, int Kmax, int V, int W,
                                          int VR, int warp) {
  WarpSmem s;
  const size_t K = (size_t)(Kmax > 0 ? Kmax : 1);
  unsigned char* p = base;
  s.red_g = reinterpret_cast<F2*>(p);
  p += fit_align16((size_t)W * K * 8);
  s.red_l = reinterpret_cast<F2*>(p);
  p += fit_align16((size_t)W * 8);
  s.pvec = reinterpret_cast<float*>(p);
  p += 512;
  s.tape = reinterpret_cast<uint32_t*>(p);
  p += fit_align16((size_t)Lmax * 4);
  s.node_slot = reinterpret_cast<int*>(p);
  p += fit_align16((size_t)Lmax * 4);
  s.slot_node = reinterpret_cast<int*>(p);
  p += fit_align16(K * 4);
  s.red_e = reinterpret_cast<int*>(p);
  p += fit_align16((size_t)W * 4);
  s.task = reinterpret_cast<long long*>(p);
  p += 16;
  s.pcode = reinterpret_cast<uint32_t*>(p);
  p += fit_align16((size_t)Lmax * 4);
  s.psa = reinterpret_cast<uint32_t*>(p);
  p += fit_align16((size_t)Lmax * 4);
  s.psb = reinterpret_cast<uint32_t*>(p);
  p += fit_align16((size_t)Lmax * 4);
  s.pda = reinterpret_cast<uint32_t*>(p);
  p += fit_align16((size_t)Lmax * 4);
  s.pdb = reinterpret_cast<uint32_t*>(p);
  p += fit_align16((size_t)Lmax * 4);
  s.arow = reinterpret_cast<int*>(p);
  p += fit_align16((size_t)Lmax * 4);
  s.frees = reinterpret_cast<int*>(p);
  p += fit_align16((size_t)Lmax * 4);
  s.rowvar = reinterpret_cast<int*>(p);
  p += fit_align16((size_t)VR * 4);
  s.info = reinterpret_cast<int*>(p);
  p += 32;
  const WarpLayout L = warp_layout(Lmax, Imax, Amax, Kmax, V, VR);
  unsigned char* t = base + fit_shared_bytes(Lmax, Kmax, W, VR) - 128;
  t = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(t) + 127) & ~uintptr_t(127));
  s.wb = t + (size_t)warp * L.bytes;
  s.bc = reinterpret_cast<float*>(s.wb);
  s.vals = reinterpret_cast<float*>(s.wb + L.vals);
  s.adj = reinterpret_cast<float*>(s.wb + L.adj);
  s.gl = reinterpret_cast<float*>(s.wb + L.gl);
  return s;
}

// Sum of two float pairs (see F2).
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bv = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bv)), __fsub_rn(b.hi, bv));
  return F2{s, __fadd_rn(__fadd_rn(a.lo, b.lo), e)};
}

// The total of a float pair (see F2).
__device__ __forceinline__ float f2_val(F2 a) { return isfinite(a.hi) ? __fadd_rn(a.hi, a.lo) : a.hi; }

// Normalised float pairs for the search direction (Dekker's double-float
// arithmetic on the FP32 pipe, about 44 significant bits): hi is the rounded value,
// lo the remainder.  f2_norm turns a cascaded sum (see F2) into one (TwoSum of its
// parts); products use FMA for the exact product of the high parts.
__device__ __forceinline__ F2 f2_norm(F2 a) {
  if (!isfinite(a.hi)) return F2{a.hi, 0.f};
  const float s = __fadd_rn(a.hi, a.lo);
  const float bv = __fsub_rn(s, a.hi);
  return F2{s, __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bv)), __fsub_rn(a.lo, bv))};
}

__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  if (!isfinite(p)) return F2{p, 0.f};
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const float s = __fadd_rn(p, e);
  return F2{s, __fsub_rn(e, __fsub_rn(s, p))};
}

__device__ __forceinline__ F2 f2_sub(F2 a, F2 b) { return f2_norm(f2_add(a, F2{-b.hi, -b.lo})); }

// a / b for normalised pairs (one float division, the remainder by FMA, a second
// division for the correction).
__device__ __forceinline__ F2 f2_div(F2 a, F2 b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  if (!isfinite(q1)) return F2{q1, 0.f};
  const float ph = __fmul_rn(q1, b.hi);
  const float pl = __fmaf_rn(q1, b.hi, -ph);
  float r = __fsub_rn(__fsub_rn(a.hi, ph), pl);
  r = __fmaf_rn(-q1, b.lo, __fadd_rn(r, a.lo));
  const float q2 = __fdiv_rn(r, b.hi);
  const float sum = __fadd_rn(q1, q2);
  return F2{sum, __fsub_rn(q2, __fsub_rn(sum, q1))};
}

__device__ __forceinline__ F2 f2_of_double(double d) {
  const float hi = __double2float_rn(d);
  return F2{hi, isfinite(hi) ? __double2float_rn(__dsub_rn(d, (double)hi)) : 0.f};
}

__device__ __forceinline__ F2 warp_sum_f2(float v) {
  F2 a{v, 0.f};
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const F2 b{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
    a = f2_add(a, b);
  }
  return a;
}

// Parameter-slot vectors: slot j lives in lane j % 32, register j / 32.
template <int SPL>
struct Slots {
  float v[SPL];
};

template <int SPL>
struct Problem {
  int64_t b;
  int root;       // index of the root node
  int K;          // real slots
  int nslots;     // K + (has virtual slot)
  bool has_virtual;
  int lane;
  __device__ __forceinline__ bool active(int s) const { return s * 32 + lane < nslots; }
  __device__ __forceinline__ bool real(int s) const { return s * 32 + lane < K; }
};

// Dot product of two slot vectors as a normalised float pair (TwoProduct by FMA,
// cascaded pair sums); every lane gets it.  With one slot per lane and at most 16
// slots, only the lanes below the next power of two hold terms, so the butterfly
// stops there and lane 0's total is broadcast.
template <int SPL>
__device__ __forceinline__ F2 dot_pair(const Problem<SPL>& P, const Slots<SPL>& a, const Slots<SPL>& b) {
  F2 acc{0.f, 0.f};
#pragma unroll
  for (int s = 0; s < SPL; ++s) {
    if (P.active(s)) {
      const float pr = __fmul_rn(a.v[s], b.v[s]);
      acc = f2_add(acc, F2{pr, __fmaf_rn(a.v[s], b.v[s], -pr)});
    }
  }
  if (SPL == 1 && P.nslots <= 16) {
    const int width = P.nslots <= 4 ? 4 : (P.nslots <= 8 ? 8 : 16);
    for (int o = width >> 1; o > 0; o >>= 1) {
      const F2 t{__shfl_xor_sync(0xffffffffu, acc.hi, o), __shfl_xor_sync(0xffffffffu, acc.lo, o)};
      acc = f2_add(acc, t);
    }
    acc = F2{__shfl_sync(0xffffffffu, acc.hi, 0), __shfl_sync(0xffffffffu, acc.lo, 0)};
  } else {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const F2 t{__shfl_xor_sync(0xffffffffu, acc.hi, o), __shfl_xor_sync(0xffffffffu, acc.lo, o)};
      acc = f2_add(acc, t);
    }
  }
  return f2_norm(acc);
}

// Dot product of two slot vectors with float-pair accumulation (TwoProduct by
// FMA, then pair sums: Ogita, Rump and Oishi's Dot2), as accurate as a dot in twice
// the precision on the FP32 pipe, rounded to float.  Used for the line-search slope
// g.p and the gradient norm; the curvature dots of the direction are kept as
// normalised pairs (dot_pair, f2_madf).
template <int SPL>
__device__ __forceinline__ float dot_f2(const Problem<SPL>& P, const Slots<SPL>& a, const Slots<SPL>& b) {
  F2 acc{0.f, 0.f};
#pragma unroll
  for (int s = 0; s < SPL; ++s) {
    if (P.active(s)) {
      const float pr = __fmul_rn(a.v[s], b.v[s]);
      acc = f2_add(acc, F2{pr, __fmaf_rn(a.v[s], b.v[s], -pr)});
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const F2 t{__shfl_xor_sync(0xffffffffu, acc.hi, o), __shfl_xor_sync(0xffffffffu, acc.lo, o)};
    acc = f2_add(acc, t);
  }
  return f2_val(acc);
}

// x + a * p, rounded as two separate float operations (never fused), so that the
// trial point and the later update x += a*p give identical bits.
template <int SPL>
__device__ __forceinline__ Slots<SPL> axpy(const Slots<SPL>& x, float a, const Slots<SPL>& p) {
  Slots<SPL> r;
#pragma unroll
  for (int s = 0; s < SPL; ++s) r.v[s] = __fadd_rn(x.v[s], __fmul_rn(a, p.v[s]));
  return r;
}

// phi0 + (c * a) * dphi0 in float32, each operation rounded on its own as the
// reference's tensor arithmetic does.
__device__ __forceinline__ float armijo(float phi0, float c, float a, float dphi0) {
  return __fadd_rn(phi0, __fmul_rn(__fmul_rn(c, a), dphi0));
}

// ---- L-BFGS history of one CTA ----
//
// Rings of the s and y vectors (hist rows of SPL*32 + 1 floats: the odd row stride
// keeps a lane per row free of bank conflicts), then float-pair words: alpha and rho
// per pair (two-loop recursion), and for histories of at most 32 pairs the compact
// representation's per-pair curvature c = s.y + eps and two hist x MS matrices (MS odd)
// indexed by ring slot: R^-1 (upper triangular in the age order) and Y^T Y.
__host__ __device__ __forceinline__ int hist_ring_stride(int SPL) { return SPL * 32 + 1; }
__host__ __device__ __forceinline__ bool hist_compact(int hist) { return hist <= 32; }
__host__ __device__ __forceinline__ int hist_mat_stride(int hist) { return hist | 1; }
__host__ __device__ __forceinline__ size_t hist_vec_bytes(int hist, int SPL) {
  return fit_align16((size_t)2 * hist * hist_ring_stride(SPL) * sizeof(float));
}
__host__ __device__ __forceinline__ size_t hist_block_bytes(int hist, int SPL) {
  const size_t words = (size_t)2 * hist + (hist_compact(hist) ? (size_t)hist + 2 * (size_t)hist * hist_mat_stride(hist) : 0);
  return hist_vec_bytes(hist, SPL) + fit_align16(words * 8);
}

struct History {
  float* S;       // [hist][RS]
  float* Y;       // [hist][RS]
  float2* alph;   // [hist] alpha of the current direction, by position (two-loop)
  float2* rho;    // [hist] 1 / c, by slot
  float2* c;      // [hist] s.y + eps, by slot (compact)
  float2* Rinv;   // [hist][MS] (compact)
  float2* YY;     // [hist][MS] (compact)
  int hist, RS, MS;
  bool compact;
  bool split;     // two lanes per pair (histories of at most 16 pairs, one slot register)
};

template <int SPL>
__device__ __forceinline__ History history_at(unsigned char* base, int hist) {
  History H;
  H.hist = hist;
  H.RS = hist_ring_stride(SPL);
  H.MS = hist_mat_stride(hist);
  H.compact = hist_compact(hist);
  H.split = SPL == 1 && hist <= 16;
  H.S = reinterpret_cast<float*>(base);
  H.Y = H.S + (size_t)hist * H.RS;
  H.alph = reinterpret_cast<float2*>(base + hist_vec_bytes(hist, SPL));
  H.rho = H.alph + hist;
  H.c = H.rho + hist;
  H.Rinv = H.c + hist;
  H.YY = H.Rinv + (size_t)hist * H.MS;
  return H;
}

// Ring slot of position j (j < hist) for the oldest pair at head (head < hist).
__device__ __forceinline__ int ring_slot(int head, int j, int hist) {
  const int s = head + j;
  return s >= hist ? s - hist : s;
}

__device__ __forceinline__ F2 ld2(const float2* p) {
  const float2 v = *p;
  return F2{v.x, v.y};
}
__device__ __forceinline__ void st2(float2* p, F2 v) { *p = make_float2(v.hi, v.lo); }
__device__ __forceinline__ F2 shfl2(F2 v, int src) {
  return F2{__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
}

// acc + a * b for float pairs: the exact product of the high parts (FMA) plus the
// cross terms, added as a cascaded pair sum (normalise the total with f2_norm).
__device__ __forceinline__ F2 f2_mad(F2 acc, F2 a, F2 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return f2_add(acc, F2{p, e});
}

// acc + a * b for floats (TwoProduct by FMA), as a cascaded pair sum.
__device__ __forceinline__ F2 f2_madf(F2 acc, float a, float b) {
  const float p = __fmul_rn(a, b);
  return f2_add(acc, F2{p, __fmaf_rn(a, b, -p)});
}

// Compact representation of the L-BFGS inverse Hessian (Byrd, Nocedal and Schnabel,
// "Representations of quasi-Newton matrices and their use in limited memory methods",
// Math. Programming 63, 1994): with the pairs (s_i, y_i) oldest first, R upper
// triangular with R_ij = s_i.y_j (i < j) and R_ii = c_i = s_i.y_i + eps, C = diag(c),
// gamma = s.y / (y.y + eps) of the newest pair,
//   H g = gamma g + S z - gamma Y t,   t = R^-1 S^T g,   z = R^-T (C t + gamma Y^T Y t - gamma Y^T g),
// which equals the two-loop recursion with rho_i = 1 / c_i.  R^-1 is kept instead of R:
// appending a pair adds the column -R^-1 r / c_new (r_i = s_i.y_new), and dropping the
// oldest pair keeps the trailing block, which is the inverse of R's trailing block.  Lane i
// of warp 0 works on the pair at position i, so every dot and every product with R^-1 or
// Y^T Y is a chain of float-pair multiply-adds on one lane, without cross-lane reductions;
// the vector is formed per slot in float.  Positions j < h, ring slot (head + j) % hist.

// The sums below run over blocks of 4 terms: the block's shared-memory loads and
// shuffles are issued first, then its 4 multiply-adds in order, masked by selects (no
// branch), so that the latencies of the loads overlap.  For histories of at most 16 pairs
// (and one slot register) two lanes work on each pair, lane i and lane i + 16 for the
// pair at position i: a sum over n terms is split into its first (n + 1) / 2 terms, summed
// in order by the lower lane, and the rest, summed in order by the upper lane, and the
// two partial sums are added (f2_add, the same in both lanes); otherwise lane i sums all
// n terms in order.

// The lane's part of a sum over n terms: terms [lo, hi), trips = loop length (the same
// in every lane).
struct SumPart {
  int lo, hi, trips;
};
__device__ __forceinline__ SumPart sum_part(bool split, int grp, int n) {
  if (!split) return SumPart{0, n, n};
  const int mid = (n + 1) >> 1;
  return grp ? SumPart{mid, n, mid} : SumPart{0, mid, mid};
}
__device__ __forceinline__ F2 join_parts(bool split, F2 a) {
  if (!split) return a;
  return f2_add(a, F2{__shfl_xor_sync(0xffffffffu, a.hi, 16), __shfl_xor_sync(0xffffffffu, a.lo, 16)});
}

// Pair position i of the lane (mine: i < h): sum over the positions j < h (kUpper:
// j >= i, kLower: j <= i) of M(i, j) x_j, x_j from lane j; M(i, j) at base + slot(j) * stride.
template <bool kUpper, bool kLower>
__device__ __forceinline__ F2 compact_matvec(const float2* base, int stride, int head, int h, int hist, F2 x,
                                             bool mine, int i, bool split, int grp) {
  F2 acc{0.f, 0.f};
  const SumPart sp = sum_part(split, grp, h);
  for (int j0 = 0; j0 < sp.trips; j0 += 4) {
    F2 xj[4], m[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int j = min(sp.lo + j0 + k, h - 1);
      xj[k] = shfl2(x, j);
      m[k] = ld2(base + (size_t)ring_slot(head, j, hist) * stride);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int j = sp.lo + j0 + k;
      const F2 n = f2_mad(acc, m[k], xj[k]);
      acc = (mine && j < sp.hi && (!kUpper || i <= j) && (!kLower || j <= i)) ? n : acc;
    }
  }
  return f2_norm(join_parts(split, acc));
}

// The history update for the newest pair (already in its ring slot, at position h - 1)
// and the direction q = H g that follows it, by the compact representation (h >= 1).
// The update is done here, not when the pair is stored: the next direction is the only
// reader, so its dots share one pass over the ring with the direction's (four chains on
// the same loads: s_i.y_new, y_i.y_new, s_i.g, y_i.g) and the new column of R^-1 shares
// the loop of t = R^-1 u.  Every sum keeps the order of its terms.  Writes c, rho, the
// row and column of Y^T Y and the column of R^-1 of the new pair, and returns s.y and
// y.y of the new pair in sy, yy (every lane).
template <int SPL>
__device__ __forceinline__ void compact_update_direction(const History& H, int head, int h, int nslots, F2 eps2,
                                                         const Slots<SPL>& g, Slots<SPL>& q, F2& sy, F2& yy,
                                                         int lane) {
  __syncwarp();  // the new pair's ring rows, written by every lane
  const bool split = H.split;
  const int grp = split ? lane >> 4 : 0;
  const int i = split ? lane & 15 : lane;  // the lane's pair position
  const bool mine = i < h;
  const int sl = mine ? ring_slot(head, i, H.hist) : 0;
  const int slot = ring_slot(head, h - 1, H.hist);
  const float* si = H.S + (size_t)sl * H.RS;
  const float* yi = H.Y + (size_t)sl * H.RS;
  const float* yn = H.Y + (size_t)slot * H.RS;
  // r_i = s_i.y_new, e_i = y_i.y_new (update); u_i = s_i.g, w_i = y_i.g (direction)
  F2 r{0.f, 0.f}, e{0.f, 0.f}, u{0.f, 0.f}, w{0.f, 0.f};
#pragma unroll
  for (int s = 0; s < SPL; ++s) {
    const int top = min(32, nslots - s * 32);
    const SumPart sp = sum_part(split, grp, top);  // split only with one slot register
    for (int l0 = 0; l0 < sp.trips; l0 += 4) {
      float gj[4], a[4], b[4], c[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int l = min(sp.lo + l0 + k, top - 1);
        gj[k] = __shfl_sync(0xffffffffu, g.v[s], l);
        a[k] = si[s * 32 + l];
        b[k] = yi[s * 32 + l];
        c[k] = yn[s * 32 + l];
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const F2 nr = f2_madf(r, a[k], c[k]), ne = f2_madf(e, b[k], c[k]);
        const F2 nu = f2_madf(u, a[k], gj[k]), nw = f2_madf(w, b[k], gj[k]);
        const bool ok = sp.lo + l0 + k < sp.hi;
        r = ok ? nr : r;
        e = ok ? ne : e;
        u = ok ? nu : u;
        w = ok ? nw : w;
      }
    }
  }
  r = f2_norm(join_parts(split, r));
  e = f2_norm(join_parts(split, e));
  u = f2_norm(join_parts(split, u));
  w = f2_norm(join_parts(split, w));
  sy = shfl2(r, h - 1);
  yy = shfl2(e, h - 1);
  const F2 cn = f2_norm(f2_add(sy, eps2));
  const F2 rho = f2_div(F2{1.f, 0.f}, cn);
  // over the older pairs (i <= j < h - 1): the new column's sum R^-1 r and t = R^-1 u
  F2 acc{0.f, 0.f}, t{0.f, 0.f};
  const float2* rrow = H.Rinv + (size_t)sl * H.MS;
  const SumPart tp = sum_part(split, grp, h - 1);
  for (int j0 = 0; j0 < tp.trips; j0 += 4) {
    F2 rj[4], uj[4], m[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int j = min(tp.lo + j0 + k, h - 2);
      rj[k] = shfl2(r, j);
      uj[k] = shfl2(u, j);
      m[k] = ld2(rrow + ring_slot(head, j, H.hist));
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int j = tp.lo + j0 + k;
      const F2 na = f2_mad(acc, m[k], rj[k]), nt = f2_mad(t, m[k], uj[k]);
      const bool ok = i <= j && j < tp.hi;
      acc = ok ? na : acc;
      t = ok ? nt : t;
    }
  }
  acc = join_parts(split, acc);
  t = join_parts(split, t);
  // the new pair's column of R^-1 (rho on the diagonal), and the last term of t
  const F2 col = f2_mul(rho, f2_norm(acc));
  const F2 rnew = i == h - 1 ? rho : F2{-col.hi, -col.lo};
  const F2 ulast = shfl2(u, h - 1);
  t = mine ? f2_mad(t, rnew, ulast) : t;
  t = f2_norm(t);
  if (mine && grp == 0) {
    st2(H.YY + (size_t)sl * H.MS + slot, e);
    st2(H.YY + (size_t)slot * H.MS + sl, e);
    st2(H.Rinv + (size_t)sl * H.MS + slot, rnew);
  }
  if (lane == 0) {
    st2(H.rho + slot, rho);
    st2(H.c + slot, cn);
  }
  __syncwarp();
  const F2 gam = f2_div(sy, f2_norm(f2_add(yy, eps2)));
  // Y^T Y t, v = c t + gamma (Y^T Y t - w), z = R^-T v (positions j <= i)
  const F2 yt =
      compact_matvec<false, false>(H.YY + (size_t)sl * H.MS, 1, head, h, H.hist, t, mine, i, split, grp);
  const F2 v = f2_norm(f2_add(f2_mul(ld2(H.c + sl), t), f2_mul(gam, f2_sub(yt, w))));
  const F2 z = compact_matvec<false, true>(H.Rinv + sl, H.MS, head, h, H.hist, v, mine, i, split, grp);
  const F2 b = f2_mul(gam, t);
  // q = gamma g + sum_i z_i s_i - sum_i (gamma t_i) y_i, per slot in float
  Slots<SPL> qs, qy;
#pragma unroll
  for (int s = 0; s < SPL; ++s) {
    qs.v[s] = __fmaf_rn(g.v[s], gam.lo, __fmul_rn(g.v[s], gam.hi));
    qy.v[s] = 0.f;
  }
  for (int i0 = 0; i0 < h; i0 += 4) {
    F2 zi[4], bi[4];
    float sv[4][SPL], yv[4][SPL];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = min(i0 + k, h - 1);
      zi[k] = shfl2(z, i);
      bi[k] = shfl2(b, i);
      const int sli = ring_slot(head, i, H.hist);
#pragma unroll
      for (int s = 0; s < SPL; ++s) {
        sv[k][s] = H.S[(size_t)sli * H.RS + s * 32 + lane];
        yv[k][s] = H.Y[(size_t)sli * H.RS + s * 32 + lane];
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const bool ok = i0 + k < h;
#pragma unroll
      for (int s = 0; s < SPL; ++s) {
        const float ns = __fmaf_rn(zi[k].lo, sv[k][s], __fmaf_rn(zi[k].hi, sv[k][s], qs.v[s]));
        const float ny = __fmaf_rn(bi[k].lo, yv[k][s], __fmaf_rn(bi[k].hi, yv[k][s], qy.v[s]));
        qs.v[s] = ok ? ns : qs.v[s];
        qy.v[s] = ok ? ny : qy.v[s];
      }
    }
  }
#pragma unroll
  for (int s = 0; s < SPL; ++s) q.v[s] = __fsub_rn(qs.v[s], qy.v[s]);
}

constexpr int kMaxRegVars = 4;  // X rows of up to this many variables are held in registers

// Value of variable `var` at the lane's point: from registers when n_x is small.
template <int V>
__device__ __forceinline__ float var_value(const float (&xr)[V][kMaxRegVars], int v, int var, bool in_regs,
                                           const float* __restrict__ X, int64_t nn, int64_t n_x) {
  if (in_regs) {
    float r = xr[v][0];
    r = var == 1 ? xr[v][1] : r;
    r = var == 2 ? xr[v][2] : r;
    r = var == 3 ? xr[v][3] : r;
    return r;
  }
  return __ldg(X + nn * n_x + var);
}

// ---------------------------------------------------------------------------------
// Operator-node program.  Before the first closure of a problem its tape (nodes up
// to the root) is rewritten as a list of operator nodes (arity >= 1, plus NO_OP
// nodes, whose value NaN and adjoint check matter).  Leaves are not executed: every
// operand is a precomputed address in the warp's table,
//   source word  = byte offset (bits 0..23) | lane stride in bytes (bits 24..31):
//                  an operator node's row or a variable's row (stride 4: one value
//                  per lane and point) or a broadcast entry (stride 0: 0, a
//                  constant slot, a fixed constant),
//   destination  = byte offset of the row that receives the operand's adjoint: the
//                  operator node's adjoint row, the constant slot's partial-sum
//                  row, or a sink row for variables and fixed constants.
// So the interpreter fetches and stores operands without branching on their kind;
// only the opcode dispatch remains (warp-uniform).
// ---------------------------------------------------------------------------------
__device__ __forceinline__ bool is_operator_node(int code) { return code == NO_OP || arity_of(code) >= 1; }

__device__ __forceinline__ bool is_fixed_leaf(int code) { return code >= C1 && code <= E_; }

// Source word and destination of operand node c (operator row / slot / variable row
// numbers in node_slot).
__device__ __forceinline__ void operand_words(const uint32_t* tape, const int* node_slot, const int* arow, int c,
                                              int Kmax, int Imax, const WarpLayout& L, uint32_t RW, uint32_t& src,
                                              uint32_t& dst) {
  const int code = code_of(tape[c]);
  if (is_operator_node(code)) {
    src = (L.vals + (uint32_t)node_slot[c] * RW) | (4u << 24);
    dst = L.adj + (uint32_t)arow[node_slot[c]] * RW;
  } else if (code == VAR) {
    src = (L.vals + (uint32_t)(Imax + node_slot[c]) * RW) | (4u << 24);
    dst = L.sink;
  } else if (code == LEARNABLE) {
    src = 4u * (1u + (uint32_t)node_slot[c]);
    dst = L.gl + (uint32_t)node_slot[c] * RW;
  } else if (is_fixed_leaf(code)) {
    src = 4u * (1u + (uint32_t)Kmax + (uint32_t)c);
    dst = L.sink;
  } else {
    src = 0u;  // the zero entry
    dst = L.sink;
  }
}

template <int V>
__device__ __forceinline__ float lds_src(const unsigned char* wb, uint32_t w, int li) {
  return *reinterpret_cast<const float*>(wb + (w & 0xffffffu) + (uint32_t)li * (w >> 24));
}

__device__ __forceinline__ float* row_ptr(unsigned char* wb, uint32_t off, int li) {
  return reinterpret_cast<float*>(wb + off) + li;
}

// ---------------------------------------------------------------------------------
// One pass over the problem's points at the constants in the warp's broadcast
// entries.  kPassGrad: loss + gradient (forward, residual, reverse sweep);
// kPassYFinal: forward only, writing the root values to Y_final; kPassLoss: forward
// and residuals only (the loss of a candidate start).  Adjoint contributions are
// added in the reference's order (parents from the last to the first, child 0
// before child 1).
// ---------------------------------------------------------------------------------
enum PassMode : int { kPassGrad = 0, kPassYFinal = 1, kPassLoss = 2 };

template <int V, int kMode>
__device__ __forceinline__ float tape_pass(const FitArgs& A, const WarpSmem& S, int64_t b, int lane, int warp, int W,
                                            int& err) {
  const int64_t N = A.N;
  const float invN = 1.0f / (float)N;
  const float* __restrict__ Yrow = A.Y ? A.Y + b * N : nullptr;
  const bool xin = A.n_x <= kMaxRegVars;
  const int nI = S.info[0];              // operator nodes
  const int root_row = S.info[1];        // the root's adjoint row, or -1 for a leaf root
  const int nvr = S.info[2];             // variable rows in use
  const uint32_t root_src = (uint32_t)S.info[3], root_dst = (uint32_t)S.info[4];
  const uint32_t sink = (uint32_t)S.info[5];  // adjoints of variables and fixed constants go nowhere
  const uint32_t RW = 32u * V;           // floats per row
  unsigned char* wb = S.wb;
  // per-lane partial sums in float (a lane sees N / (32 V W) points)
  float loss_part = 0.f;
  for (int64_t base = (int64_t)warp * 32 * V; base < N; base += (int64_t)W * 32 * V) {
    int64_t nn[V];
    bool valid[V];
    float xr[V][kMaxRegVars];
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const int64_t n = base + v * 32 + lane;
      valid[v] = n < N;
      nn[v] = valid[v] ? n : N - 1;
#pragma unroll
      for (int j = 0; j < kMaxRegVars; ++j) xr[v][j] = (xin && j < A.n_x) ? __ldg(A.X + nn[v] * A.n_x + j) : 0.f;
    }
    // variable rows of this chunk
    for (int r = 0; r < nvr; ++r) {
      const int var = S.rowvar[r];
#pragma unroll
      for (int v = 0; v < V; ++v)
        S.vals[(A.Imax + r) * RW + v * 32 + lane] = var_value<V>(xr, v, var, xin, A.X, nn[v], A.n_x);
    }
    __syncwarp();
    // ---- forward over the operator nodes ----
    uint32_t cn = nI > 0 ? S.pcode[0] : 0u, san = nI > 0 ? S.psa[0] : 0u, sbn = nI > 0 ? S.psb[0] : 0u;
    for (int i = 0; i < nI; ++i) {
      const int code = (int)(cn & 0xffu);
      const uint32_t sa = san, sb = sbn;
      if (i + 1 < nI) {
        cn = S.pcode[i + 1];
        san = S.psa[i + 1];
        sbn = S.psb[i + 1];
      }
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const int li = v * 32 + lane;
        const float r = op_value<float>(code, lds_src<V>(wb, sa, li), lds_src<V>(wb, sb, li));
        S.vals[i * RW + li] = r;
      }
    }
    float fval[V];
#pragma unroll
    for (int v = 0; v < V; ++v) fval[v] = lds_src<V>(wb, root_src, v * 32 + lane);
    if constexpr (kMode == kPassYFinal) {
#pragma unroll
      for (int v = 0; v < V; ++v)
        if (valid[v]) A.Y_final[b * N + nn[v]] = fval[v];
      __syncwarp();
      continue;
    } else if constexpr (kMode == kPassLoss) {
#pragma unroll
      for (int v = 0; v < V; ++v) {
        if (valid[v]) {
          if (A.objective == 0) {
            const float rr = fval[v] - __ldg(Yrow + nn[v]);
            loss_part = __fadd_rn(loss_part, __fmul_rn(rr, rr));
          } else {
            loss_part = __fadd_rn(loss_part, fval[v]);
          }
        }
      }
      __syncwarp();
      continue;
    } else {
    // ---- residuals: root adjoint (2 (f - y)) * (1/N), as autograd forms it ----
#pragma unroll
    for (int v = 0; v < V; ++v) {
      float groot = 0.f;
      if (valid[v]) {
        if (A.objective == 0) {
          const float rr = fval[v] - __ldg(Yrow + nn[v]);
          loss_part = __fadd_rn(loss_part, __fmul_rn(rr, rr));
          groot = __fmul_rn(rr * 2.0f, invN);
        } else {
          loss_part = __fadd_rn(loss_part, fval[v]);
          groot = invN;
        }
      }
      const int li = v * 32 + lane;
      if (root_row >= 0) {
        S.adj[root_row * RW + li] = groot;  // the seed of the root (its row holds 0)
      } else if (groot != 0.f) {
        float* d = row_ptr(wb, root_dst, li);  // a leaf root: its slot's row, or the sink
        *d = __fadd_rn(*d, groot);
      }
    }
    // ---- reverse sweep over the operator nodes ----
    uint32_t cp = 0u, sap = 0u, sbp = 0u, dap = 0u, dbp = 0u;
    if (nI > 0) {
      cp = S.pcode[nI - 1]; sap = S.psa[nI - 1]; sbp = S.psb[nI - 1]; dap = S.pda[nI - 1]; dbp = S.pdb[nI - 1];
    }
    for (int i = nI - 1; i >= 0; --i) {
      const int code = (int)(cp & 0xffu);
      const uint32_t arow = (cp >> 8) * RW;  // the node's adjoint row (float offset)
      const uint32_t sa = sap, sb = sbp, da = dap, db = dbp;
      if (i > 0) {
        cp = S.pcode[i - 1]; sap = S.psa[i - 1]; sbp = S.psb[i - 1]; dap = S.pda[i - 1]; dbp = S.pdb[i - 1];
      }
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const int li = v * 32 + lane;
        const float g = S.adj[arow + li];
        S.adj[arow + li] = 0.f;  // read once: the row is free for the nodes swept next
        bool a0, a1;
        float r0, r1;
        const int e = op_adjoint<float>(code, g, lds_src<V>(wb, sa, li), lds_src<V>(wb, sb, li), S.vals[i * RW + li],
                                          a0, r0, a1, r1);
        if (valid[v]) {
          if (e && !err) err = e;
          if (a0 && da != sink) {
            float* d = row_ptr(wb, da, li);
            *d = __fadd_rn(*d, r0);
          }
          if (a1 && db != sink) {
            float* d = row_ptr(wb, db, li);
            *d = __fadd_rn(*d, r1);
          }
        }
      }
    }
    __syncwarp();
    }  // kPassGrad
  }
  return loss_part;
}

// Sums over the 32 lanes of KP per-lane values at once (the per-slot gradient
// partials and the loss partial) by recursive halving: at each step a lane keeps
// half of its values and receives its partner's partial sums of that half, so KP
// values need KP - 1 + 5 - log2(KP) pair exchanges instead of 5 KP.  Every slot's
// total ends in the lanes whose high bits spell it; f2_add does not depend on the
// operand order, so the result is deterministic.
template <int KP>
__device__ __forceinline__ void reduce_slots(const float* __restrict__ gl, int V, int K, float loss_part, int lane,
                                             F2* __restrict__ out_g, F2* __restrict__ out_l) {
  F2 x[KP];
#pragma unroll
  for (int j = 0; j < KP; ++j) {
    float part = 0.f;
    if (j < K) {
      part = gl[j * 32 * V + lane];
      for (int v = 1; v < V; ++v) part = __fadd_rn(part, gl[j * 32 * V + v * 32 + lane]);
    } else if (j == K) {
      part = loss_part;
    }
    x[j] = F2{part, 0.f};
  }
  int slot = 0;
  int n = KP;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    if (n > 1) {
      const bool up = (lane & o) != 0;
      const int h = n >> 1;
#pragma unroll
      for (int t = 0; t < KP / 2; ++t) {
        if (t < h) {
          const F2 send = up ? x[t] : x[t + h];
          const F2 keep = up ? x[t + h] : x[t];
          const F2 recv{__shfl_xor_sync(0xffffffffu, send.hi, o), __shfl_xor_sync(0xffffffffu, send.lo, o)};
          x[t] = f2_add(keep, recv);
        }
      }
      slot = slot * 2 + (up ? 1 : 0);
      n = h;
    } else {
      const F2 recv{__shfl_xor_sync(0xffffffffu, x[0].hi, o), __shfl_xor_sync(0xffffffffu, x[0].lo, o)};
      x[0] = f2_add(x[0], recv);
    }
  }
  // lanes with the same high bits hold the same total: the lowest of them writes it
  constexpr int kGroup = 32 / KP;
  if ((lane & (kGroup - 1)) == 0) {
    if (slot < K) out_g[slot] = x[0];
    else if (slot == K) *out_l = x[0];
  }
}

// Closure: publish the trial constants, run the pass over this warp's points,
// reduce loss and gradient over the lanes (recursive halving) and then over the CTA's
// warps in a fixed order, in float pairs on the FP32 pipe (GB300's FP64 rate is a
// small fraction of its FP32 rate); every warp ends with the same bits.  Two CTA
// barriers.
template <int V, int SPL>
__device__ __forceinline__ float closure(const FitArgs& A, const WarpSmem& S, const Problem<SPL>& P, int warp, int W,
                                         const Slots<SPL>& xt, Slots<SPL>& grad, int& err) {
  const int lane = P.lane;
  // every warp holds the same trial point: each publishes it into its own broadcast entries
#pragma unroll
  for (int s = 0; s < SPL; ++s)
    if (P.real(s)) S.bc[1 + s * 32 + lane] = xt.v[s];
  for (int j = 0; j < P.K; ++j) {
#pragma unroll
    for (int v = 0; v < V; ++v) S.gl[j * 32 * V + v * 32 + lane] = 0.f;
  }
  __syncthreads();  // also: every warp has read the previous closure's reduction buffers
  const float lpart = tape_pass<V, kPassGrad>(A, S, P.b, lane, warp, W, err);
  F2* out_g = S.red_g + warp * P.K;
  if (P.K < 32) {
    if (P.K < 1) reduce_slots<1>(S.gl, V, P.K, lpart, lane, out_g, S.red_l + warp);
    else if (P.K < 2) reduce_slots<2>(S.gl, V, P.K, lpart, lane, out_g, S.red_l + warp);
    else if (P.K < 4) reduce_slots<4>(S.gl, V, P.K, lpart, lane, out_g, S.red_l + warp);
    else if (P.K < 8) reduce_slots<8>(S.gl, V, P.K, lpart, lane, out_g, S.red_l + warp);
    else if (P.K < 16) reduce_slots<16>(S.gl, V, P.K, lpart, lane, out_g, S.red_l + warp);
    else reduce_slots<32>(S.gl, V, P.K, lpart, lane, out_g, S.red_l + warp);
  } else {
    const F2 lsum = warp_sum_f2(lpart);
    for (int j = 0; j < P.K; ++j) {
      float part = S.gl[j * 32 * V + lane];
#pragma unroll
      for (int v = 1; v < V; ++v) part = __fadd_rn(part, S.gl[j * 32 * V + v * 32 + lane]);
      const F2 t = warp_sum_f2(part);
      if (lane == 0) out_g[j] = t;
    }
    if (lane == 0) S.red_l[warp] = lsum;
  }
  __syncthreads();
#pragma unroll
  for (int s = 0; s < SPL; ++s) {
    F2 acc{0.f, 0.f};
    if (P.real(s)) {
      const int j = s * 32 + lane;
      for (int w = 0; w < W; ++w) acc = f2_add(acc, S.red_g[w * P.K + j]);
    }
    grad.v[s] = f2_val(acc);
  }
  F2 lt{0.f, 0.f};
  for (int w = 0; w < W; ++w) lt = f2_add(lt, S.red_l[w]);
  return __fdiv_rn(f2_val(lt), (float)A.N);
}

// Evaluated point: value and gradient.
template <int SPL>
struct Point {
  float phi;
  Slots<SPL> g;
};

// Status of a tape larger than the tables the launch was sized for (its root + 1
// above max_len, its constants above max_consts or its operator nodes above
// max_operators): the problem is skipped before it touches shared memory.
constexpr int kStatusTapeExceedsLaunch = 602;

// Whether problem b fits the launch's tables: counted by every warp from the node
// words in global memory, so the answer is the same in every thread of the CTA.
__device__ __forceinline__ bool problem_fits(const FitArgs& A, int64_t b, int L, int K, int lane) {
  if (L < 1 || L > A.Lmax || K < 0 || K > (A.Kmax > 0 ? A.Kmax : 0)) return false;
  int nop = 0;
  for (int k0 = 0; k0 < L; k0 += 32) {
    const int k = k0 + lane;
    const bool opn = k < L && is_operator_node(code_of(A.desc[b * A.M + k]));
    nop += __popc(__ballot_sync(0xffffffffu, opn));
  }
  return nop <= A.Imax;
}

// Stages problem b (a tape of L = root + 1 nodes) for the CTA: the tape, the numbering
// of its constant slots, operator nodes and variables, the adjoint rows by liveness,
// the operator-node program (warp 0), then every warp's broadcast entries (0 and the
// fixed constants) and zeroed adjoint rows.  Ends with the tables visible to the CTA;
// false when the tape needs more live adjoint rows than the launch's max_live.
template <int V>
__device__ __forceinline__ bool stage_problem(const FitArgs& A, const WarpSmem& S, int64_t b, int L, int lane,
                                              int warp) {
  // stage the tape; number the constant slots, the operator nodes and the
  // variables; write the operator-node program (warp 0), visible to the CTA
  if (warp == 0) {
    for (int k = lane; k < L; k += 32) S.tape[k] = A.desc[b * A.M + k];
    __syncwarp();
    int nslot = 0, nop = 0;
    for (int k0 = 0; k0 < L; k0 += 32) {
      const int k = k0 + lane;
      const int code = k < L ? code_of(S.tape[k]) : -1;
      const bool lc = code == LEARNABLE;
      const bool opn = k < L && is_operator_node(code);
      const unsigned mc = __ballot_sync(0xffffffffu, lc);
      const unsigned mo = __ballot_sync(0xffffffffu, opn);
      const unsigned below = (1u << lane) - 1u;
      if (lc) {
        const int slot = nslot + __popc(mc & below);
        S.node_slot[k] = slot;
        S.slot_node[slot] = k;
      }
      if (opn) S.node_slot[k] = nop + __popc(mo & below);
      nslot += __popc(mc);
      nop += __popc(mo);
    }
    if (lane == 0) {  // one row per distinct variable, in order of first use
      int nvr = 0;
      for (int k = 0; k < L; ++k) {
        const uint32_t d = S.tape[k];
        if (code_of(d) != VAR) continue;
        const int var = child0(d);
        int r = 0;
        while (r < nvr && S.rowvar[r] != var) ++r;
        if (r == nvr) S.rowvar[nvr++] = var;
        S.node_slot[k] = r;
      }
      S.info[2] = nvr;
      // adjoint rows by liveness: an operator node holds a row from the sweep of its
      // first parent (the root from the start) to its own sweep, then frees it; rows
      // are taken from a stack, so the assignment is the same in every run
      int top = 0;
      for (int r = A.Amax - 1; r >= 0; --r) S.frees[top++] = r;
      for (int i = 0; i < nop; ++i) S.arow[i] = -1;
      bool over = false;
      const int R = L - 1;
      if (is_operator_node(code_of(S.tape[R]))) {
        if (top > 0) S.arow[S.node_slot[R]] = S.frees[--top];
        else over = true;
      }
      for (int k = R; k >= 0 && !over; --k) {
        const uint32_t d = S.tape[k];
        const int code = code_of(d);
        if (!is_operator_node(code)) continue;
        const int i = S.node_slot[k];
        if (S.arow[i] < 0) {  // no parent: a zero row for the length of its own sweep
          if (top == 0) { over = true; break; }
          S.arow[i] = S.frees[--top];
        }
        S.frees[top++] = S.arow[i];
        const int ar = arity_of(code);
        for (int j = 0; j < ar && !over; ++j) {
          const int c = j == 0 ? child0(d) : child1(d);
          if (!is_operator_node(code_of(S.tape[c])) || S.arow[S.node_slot[c]] >= 0) continue;
          if (top == 0) { over = true; break; }
          S.arow[S.node_slot[c]] = S.frees[--top];
        }
      }
      S.info[6] = over ? 1 : 0;
    }
    __syncwarp();
    const WarpLayout WL = warp_layout(A.Lmax, A.Imax, A.Amax, A.Kmax, V, A.VR);
    const uint32_t RWB = 32u * V * 4u;
    for (int k = lane; k < L; k += 32) {
      const uint32_t d = S.tape[k];
      const int code = code_of(d);
      if (!is_operator_node(code)) continue;
      const int ar = arity_of(code);
      uint32_t sa = 0u, sb = 0u, da = WL.sink, db = WL.sink;
      if (ar >= 1) operand_words(S.tape, S.node_slot, S.arow, child0(d), A.Kmax, A.Imax, WL, RWB, sa, da);
      if (ar == 2) operand_words(S.tape, S.node_slot, S.arow, child1(d), A.Kmax, A.Imax, WL, RWB, sb, db);
      const int row = S.node_slot[k];
      S.pcode[row] = (uint32_t)dense_op(code) | ((uint32_t)S.arow[row] << 8);  // opcode | adjoint row
      S.psa[row] = sa;
      S.psb[row] = sb;
      S.pda[row] = da;
      S.pdb[row] = db;
    }
    if (lane == 0) {
      const int R = (L - 1);
      uint32_t rs, rdst;
      operand_words(S.tape, S.node_slot, S.arow, R, A.Kmax, A.Imax, WL, RWB, rs, rdst);
      S.info[0] = nop;
      S.info[1] = is_operator_node(code_of(S.tape[R])) ? S.arow[S.node_slot[R]] : -1;  // the root's adjoint row
      S.info[3] = (int)rs;
      S.info[4] = (int)rdst;
      S.info[5] = (int)WL.sink;
    }
  }
  __syncthreads();
  const bool rows_suffice = S.info[6] == 0;  // written by warp 0 before the barrier
  // this warp's broadcast entries: 0 and the fixed constants of the tape
  if (lane == 0) S.bc[0] = 0.f;
  for (int k = lane; k < L; k += 32) {
    const int code = code_of(S.tape[k]);
    if (is_fixed_leaf(code)) S.bc[1 + A.Kmax + k] = node_value<float>(code, 0.f, 0.f, 0.f, 0.f);
  }
  // this warp's adjoint rows start at zero; every sweep leaves them so (a node's row is
  // reset when the node reads it)
  for (int r = 0; r < A.Amax; ++r)
    for (int v = 0; v < V; ++v) S.adj[r * 32 * V + v * 32 + lane] = 0.f;
  __syncwarp();
  return rows_suffice;
}

// Line-search phases of the per-problem state machine.  Every loop turn of the
// kernel evaluates exactly one closure (one call site, inlined), then advances the
// state; the transitions follow LBFGS_batch.step / _strong_wolfe /
// _alpha_zoom_corrected / _backtracking_line_search for one column.
enum Phase : int { PH_INIT = 0, PH_BRACKET, PH_ZOOM_LO, PH_ZOOM, PH_BACKTRACK, PH_UPDATE, PH_DONE };

template <int V, int SPL>
__global__ void __launch_bounds__(256, 2) fit_lbfgs_kernel(FitArgs A) {
  // L-BFGS constants in the iteration's arithmetic: eps as a float pair, the gradient
  // tolerance in float32 (the reference compares a float32 norm with it)
  const F2 eps2 = f2_of_double(A.eps);
  const float tolf = __double2float_rn(A.tol);
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, W = blockDim.x >> 5;
  const WarpSmem S = carve(smem, A.Lmax, A.Imax, A.Amax, A.Kmax, V, W, A.VR, warp);
  // the L-BFGS history of this CTA (used by warp 0)
  const History H = history_at<SPL>(
      A.ring_off ? smem + A.ring_off : A.ws_hist + (int64_t)blockIdx.x * (int64_t)hist_block_bytes(A.hist, SPL), A.hist);
  const float c1 = 1e-4f, c2 = 0.9f, amax = 20.0f;

  while (true) {
    // the CTA takes the next problem from the queue
    if (threadIdx.x == 0) *S.task = (long long)atomicAdd(A.counter, 1);
    __syncthreads();
    const int64_t idx = (int64_t)*S.task;
    __syncthreads();
    if (idx >= A.B) break;
    Problem<SPL> P;
    P.b = A.order ? (int64_t)A.order[idx] : idx;
    P.lane = lane;
    P.root = A.meta[P.b * 4 + 1];
    P.K = A.meta[P.b * 4 + 2];
    P.has_virtual = A.M > P.K;
    P.nslots = P.K + (P.has_virtual ? 1 : 0);
    const int L = P.root + 1;
    // a caller's max_len / max_consts / max_operators / max_live too small: not fitted
    if (!problem_fits(A, P.b, L, P.K, lane) || !stage_problem<V>(A, S, P.b, L, lane, warp)) {
      if (warp == 0) {
        const float qnan = __int_as_float(0x7fffffff);
        for (int64_t k = lane; k < A.M; k += 32) A.C_out[P.b * A.c_sb + k * A.c_sm] = A.C_init[P.b * A.c_sb + k * A.c_sm];
        if (A.Y_final)
          for (int64_t n = lane; n < A.N; n += 32) A.Y_final[P.b * A.N + n] = qnan;
        if (lane == 0) {
          report(A.status, kStatusTapeExceedsLaunch);
          if (A.iters_out) A.iters_out[P.b] = -kStatusTapeExceedsLaunch;
          if (A.loss_out) A.loss_out[P.b] = qnan;
          if (A.evals_out) A.evals_out[P.b] = 0;
        }
      }
      continue;
    }

    const float* Cin = A.C_init + P.b * A.c_sb;
    Slots<SPL> x, g, p, xn;
#pragma unroll
    for (int s = 0; s < SPL; ++s) {
      const int j = s * 32 + lane;
      x.v[s] = P.real(s) ? Cin[(int64_t)S.slot_node[j] * A.c_sm] : 0.f;
      g.v[s] = 0.f;
      p.v[s] = 0.f;
      xn.v[s] = 0.f;
    }
    int err = 0, evals = 0;
    float f = 0.f;
    bool poison = false;
    int h = 0, head = 0, it = 0;
    F2 last_sy{0.f, 0.f}, last_yy{0.f, 0.f};  // warp 0: s.y and y.y of the newest history pair
    // line-search state
    int phase = PH_INIT;
    int lsi = 0, zj = 0;
    float phi0 = 0.f, dphi0 = 0.f, a_prev = 0.f, phi_prev = 0.f, a_i = 1.f, lo = 0.f, hi = 0.f, aj = 0.f, al = 1.f;
    float alpha = 0.f;
    Point<SPL> prevpt, plo, acc;
    acc.phi = 0.f;
    prevpt.phi = 0.f;
    plo.phi = 0.f;
#pragma unroll
    for (int s = 0; s < SPL; ++s) { prevpt.g.v[s] = 0.f; plo.g.v[s] = 0.f; acc.g.v[s] = 0.f; }

    while (phase != PH_DONE) {
      // ---- trial point of this turn ----
      Slots<SPL> xt;
      switch (phase) {
        case PH_INIT: xt = x; break;
        case PH_BRACKET: xt = axpy(x, a_i, p); break;
        case PH_ZOOM_LO: xt = axpy(x, 0.f, p); break;
        case PH_ZOOM: aj = __fdiv_rn(__fadd_rn(lo, hi), 2.0f); xt = axpy(x, aj, p); break;
        case PH_BACKTRACK: xt = axpy(x, al, p); break;
        default: xt = xn; break;  // PH_UPDATE
      }
      Point<SPL> cur;
      cur.phi = closure<V, SPL>(A, S, P, warp, W, xt, cur.g, err);
      ++evals;

      // ---- advance the state machine ----
      bool ls_finished = false, known = false;
      bool begin_iter = false;
      if (phase == PH_INIT) {
        f = cur.phi;
        g = cur.g;
        begin_iter = true;
      } else if (phase == PH_BRACKET) {
        const float dphi = dot_f2(P, cur.g, p);
        const bool bad = (cur.phi > armijo(phi0, c1, a_i, dphi0)) || (lsi > 0 && cur.phi >= phi_prev);
        const bool good = fabsf(dphi) <= __fmul_rn(c2, fabsf(dphi0));
        const bool passed = dphi >= 0.f;
        if (good) {
          alpha = a_i;
          acc = cur;
          known = true;
          ls_finished = true;
        } else if (bad || passed) {
          lo = bad ? a_prev : a_i;
          hi = bad ? a_i : a_prev;
          zj = 0;
          if (!bad) {
            plo = cur;
            phase = PH_ZOOM;
          } else if (lsi > 0) {
            plo = prevpt;
            phase = PH_ZOOM;
          } else {
            // alpha_lo = 0: the point x + 0*p is x unless p holds inf/NaN
            const Slots<SPL> x0 = axpy(x, 0.f, p);
            bool same = true;
#pragma unroll
            for (int s = 0; s < SPL; ++s)
              if (P.real(s) && __float_as_uint(x0.v[s]) != __float_as_uint(x.v[s])) same = false;
            same = __all_sync(0xffffffffu, same);
            if (same) {
              plo.phi = f;
              plo.g = g;
              phase = PH_ZOOM;
            } else {
              phase = PH_ZOOM_LO;
            }
          }
        } else {
          a_prev = a_i;
          phi_prev = cur.phi;
          prevpt = cur;
          a_i = __fadd_rn(a_i, __fmul_rn(__fsub_rn(amax, a_i), 0.8f));
          ++lsi;
          if (lsi >= A.ls_max) {  // unfinished bracket: the next extrapolated step, not evaluated
            alpha = a_i;
            known = false;
            ls_finished = true;
          }
        }
      } else if (phase == PH_ZOOM_LO) {
        plo = cur;
        phase = PH_ZOOM;
      } else if (phase == PH_ZOOM) {
        const float dphij = dot_f2(P, cur.g, p);
        const bool zbad = (cur.phi > armijo(phi0, c1, aj, dphi0)) || (cur.phi >= plo.phi);
        const bool zgood = fabsf(dphij) <= __fmul_rn(c2, fabsf(dphi0));
        bool zdone = false;
        if (zgood) {
          alpha = aj;
          acc = cur;
          zdone = true;
        }
        if (!zdone) {
          const float thi = zbad ? aj : hi;
          const bool cond3 = __fmul_rn(dphij, __fsub_rn(thi, lo)) >= 0.f;
          hi = (!zbad && cond3) ? lo : thi;
          if (!zbad) {
            lo = aj;
            plo = cur;
          }
        }
        if (!zdone && fabsf(__fsub_rn(hi, lo)) < 1e-9f) {
          alpha = aj;
          acc = cur;
          zdone = true;
        }
        ++zj;
        if (!zdone && zj >= 10) {
          alpha = lo;
          acc = plo;
          zdone = true;
        }
        if (zdone) {
          known = true;
          ls_finished = true;
        }
      } else if (phase == PH_BACKTRACK) {
        if (cur.phi <= armijo(f, 1e-4f, al, dphi0)) {
          alpha = al;
          acc = cur;
          known = true;
          ls_finished = true;
        } else {
          al = al * 0.5f;
          ++lsi;
          if (lsi >= A.ls_max) {
            alpha = al;
            known = false;
            ls_finished = true;
          }
        }
      }

      // ---- end of the line search: the update x += alpha p ----
      Slots<SPL> sv;
      bool finish_iter = false;
      Point<SPL> nxt;
      if (phase == PH_UPDATE) {
        nxt = cur;
        finish_iter = true;
      } else if (ls_finished) {
#pragma unroll
        for (int s = 0; s < SPL; ++s) {
          sv.v[s] = P.active(s) ? __fmul_rn(alpha, p.v[s]) : 0.f;
          xn.v[s] = __fadd_rn(x.v[s], sv.v[s]);
        }
        if (known) {
          nxt = acc;
          finish_iter = true;
        } else {
          phase = PH_UPDATE;
        }
      }
      if (finish_iter) {
        if (phase == PH_UPDATE) {  // the step of the line search that ended in the previous turn
#pragma unroll
          for (int s = 0; s < SPL; ++s) sv.v[s] = P.active(s) ? __fmul_rn(alpha, p.v[s]) : 0.f;
        }
        if (P.has_virtual) {
          bool vnan = false;
#pragma unroll
          for (int s = 0; s < SPL; ++s)
            if (s * 32 + lane == P.K && isnan(sv.v[s])) vnan = true;
          poison = poison || __any_sync(0xffffffffu, vnan);
        }
        // push (s, y): drop the oldest pair when the history is full
        int slot;
        if (h < A.hist) {
          slot = (head + h) % A.hist;
          ++h;
        } else {
          slot = head;
          head = (head + 1) % A.hist;
        }
        if (warp == 0) {  // only warp 0 computes directions
          Slots<SPL> yv;
#pragma unroll
          for (int s = 0; s < SPL; ++s) {
            yv.v[s] = P.active(s) ? __fsub_rn(nxt.g.v[s], g.v[s]) : 0.f;
            H.S[(size_t)slot * H.RS + s * 32 + lane] = sv.v[s];
            H.Y[(size_t)slot * H.RS + s * 32 + lane] = yv.v[s];
          }
          if (!H.compact) {  // the compact form updates its history with the next direction
            // curvature of the new pair, computed once: rho of its slot, and s.y, y.y for gamma
            last_sy = dot_pair(P, yv, sv);
            last_yy = dot_pair(P, yv, yv);
            if (lane == 0) st2(H.rho + slot, f2_div(F2{1.f, 0.f}, f2_norm(f2_add(last_sy, eps2))));
          }
        }
        __syncwarp();
        x = xn;
        g = nxt.g;
        f = nxt.phi;
        ++it;
        // all real slots NaN and the others poisoned: nothing can change any more (the same in every warp)
        bool allnan = true;
#pragma unroll
        for (int s = 0; s < SPL; ++s)
          if (P.real(s) && !isnan(x.v[s])) allnan = false;
        allnan = __all_sync(0xffffffffu, allnan);
        if (P.K > 0 && allnan && (poison || !P.has_virtual)) {
          it = A.max_iter;
          phase = PH_DONE;
        } else {
          begin_iter = true;
        }
      }

      // ---- start of an outer iteration: convergence test, direction, line search ----
      if (begin_iter) {
        if (it >= A.max_iter || __fsqrt_rn(dot_f2(P, g, g)) < tolf) {
          phase = PH_DONE;
        } else {
          // direction q = H g (lbfgs_batch.py:65-103), by warp 0 for the CTA
          Slots<SPL> q = g;
          if (warp == 0 && h > 0) {
            if (H.compact) {
              compact_update_direction<SPL>(H, head, h, P.nslots, eps2, g, q, last_sy, last_yy, lane);
            } else {
              const F2 gam = f2_div(last_sy, f2_norm(f2_add(last_yy, eps2)));
              // two-loop recursion for long histories
              for (int i = h - 1; i >= 0; --i) {
                const int sl = (head + i) % A.hist;
                Slots<SPL> si, yi;
#pragma unroll
                for (int s = 0; s < SPL; ++s) {
                  si.v[s] = H.S[(size_t)sl * H.RS + s * 32 + lane];
                  yi.v[s] = H.Y[(size_t)sl * H.RS + s * 32 + lane];
                }
                // alpha = rho (s.q) and q -= alpha y: float pairs on the FP32 pipe (GB300's
                // FP64 pipe runs a warp instruction at a small fraction of the FP32 rate)
                const F2 a = f2_mul(ld2(H.rho + sl), dot_pair(P, si, q));
#pragma unroll
                for (int s = 0; s < SPL; ++s) q.v[s] = __fmaf_rn(-a.lo, yi.v[s], __fmaf_rn(-a.hi, yi.v[s], q.v[s]));
                if (lane == 0) st2(H.alph + i, a);
              }
              __syncwarp();
#pragma unroll
              for (int s = 0; s < SPL; ++s) q.v[s] = __fmaf_rn(q.v[s], gam.lo, __fmul_rn(q.v[s], gam.hi));
              for (int i = 0; i < h; ++i) {
                const int sl = (head + i) % A.hist;
                Slots<SPL> si, yi;
#pragma unroll
                for (int s = 0; s < SPL; ++s) {
                  si.v[s] = H.S[(size_t)sl * H.RS + s * 32 + lane];
                  yi.v[s] = H.Y[(size_t)sl * H.RS + s * 32 + lane];
                }
                const F2 be = f2_mul(ld2(H.rho + sl), dot_pair(P, yi, q));
                const F2 coef = f2_sub(ld2(H.alph + i), be);
#pragma unroll
                for (int s = 0; s < SPL; ++s) q.v[s] = __fmaf_rn(coef.lo, si.v[s], __fmaf_rn(coef.hi, si.v[s], q.v[s]));
              }
            }
          }
          if (warp == 0) {
#pragma unroll
            for (int s = 0; s < SPL; ++s) S.pvec[s * 32 + lane] = P.active(s) ? -q.v[s] : 0.f;
          }
          __syncthreads();
#pragma unroll
          for (int s = 0; s < SPL; ++s) p.v[s] = S.pvec[s * 32 + lane];
          phi0 = f;
          dphi0 = dot_f2(P, g, p);
          lsi = 0;
          if (A.ls_kind == 0) {
            a_prev = 0.f;
            phi_prev = phi0;
            a_i = 1.f;
            phase = PH_BRACKET;
            if (A.ls_max <= 0) {  // no bracket step: alpha = 1, not evaluated
              alpha = a_i;
#pragma unroll
              for (int s = 0; s < SPL; ++s) xn.v[s] = __fadd_rn(x.v[s], P.active(s) ? __fmul_rn(alpha, p.v[s]) : 0.f);
              phase = PH_UPDATE;
            }
          } else {
            al = 1.f;
            phase = PH_BACKTRACK;
            if (A.ls_max <= 0) {
              alpha = al;
#pragma unroll
              for (int s = 0; s < SPL; ++s) xn.v[s] = __fadd_rn(x.v[s], P.active(s) ? __fmul_rn(alpha, p.v[s]) : 0.f);
              phase = PH_UPDATE;
            }
          }
        }
      }
    }

    // errors are found per lane (per data point): combine them over the CTA
    err = __reduce_max_sync(0xffffffffu, err);
    if (lane == 0) S.red_e[warp] = err;
    __syncthreads();
    for (int w = 0; w < W; ++w) err = max(err, S.red_e[w]);
    // ---- outputs (warp 0) ----
    if (warp == 0) {
      if (err && lane == 0) report(A.status, err);
      const float qnan = __int_as_float(0x7fffffff);
      float* Cout = A.C_out + P.b * A.c_sb;
      for (int64_t k = lane; k < A.M; k += 32) Cout[k * A.c_sm] = poison ? qnan : Cin[k * A.c_sm];
      __syncwarp();
#pragma unroll
      for (int s = 0; s < SPL; ++s)
        if (P.real(s)) Cout[(int64_t)S.slot_node[s * 32 + lane] * A.c_sm] = x.v[s];
      if (lane == 0) {
        // a problem whose closures raised an error reports -code instead of its iterations
        if (A.iters_out) A.iters_out[P.b] = err ? -err : it;
        if (A.loss_out) A.loss_out[P.b] = f;
        if (A.evals_out) A.evals_out[P.b] = evals;
      }
    }
    // the final constants into every warp's broadcast entries for the Y_final pass
#pragma unroll
    for (int s = 0; s < SPL; ++s)
      if (P.real(s)) S.bc[1 + s * 32 + lane] = x.v[s];
    __syncthreads();
    if (A.Y_final) {
      int dummy = 0;
      tape_pass<V, kPassYFinal>(A, S, P.b, lane, warp, W, dummy);
    }
    __syncthreads();
  }
}

// Loss of K candidate starts per problem (multi-start screening in one launch): the
// problem's tape is staged once, then for each candidate its constants are published
// and one forward pass over the points sums the squared residuals (float per lane,
// float pairs over the lanes and then the warps in a fixed order), so
// loss_out[b, k] is the mean squared error from candidate k, as the fit's first
// closure measures it (to the last bit but for the order of the lane sum).
// Candidate k of problem b: C_sets + k c_sk + b c_sb, slot m at + m c_sm.
template <int V>
__global__ void __launch_bounds__(256, 2) fit_screen_kernel(FitArgs A, const float* __restrict__ C_sets, int64_t c_sk,
                                                            int64_t K, float* __restrict__ loss_out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, W = blockDim.x >> 5;
  const WarpSmem S = carve(smem, A.Lmax, A.Imax, A.Amax, A.Kmax, V, W, A.VR, warp);
  for (int64_t b = blockIdx.x; b < A.B; b += gridDim.x) {
    const int L = A.meta[b * 4 + 1] + 1;
    const int Kc = A.meta[b * 4 + 2];
    // a caller's max_len / max_consts / max_operators / max_live too small
    if (!problem_fits(A, b, L, Kc, lane) || !stage_problem<V>(A, S, b, L, lane, warp)) {
      if (threadIdx.x == 0) {
        report(A.status, kStatusTapeExceedsLaunch);
        for (int64_t k = 0; k < K; ++k) loss_out[b * K + k] = __int_as_float(0x7fffffff);
      }
      __syncthreads();  // the next problem's staging overwrites the tables
      continue;
    }
    for (int64_t k = 0; k < K; ++k) {
      const float* Cin = C_sets + k * c_sk + b * A.c_sb;
      for (int j = lane; j < Kc; j += 32) S.bc[1 + j] = Cin[(int64_t)S.slot_node[j] * A.c_sm];
      __syncthreads();  // also: thread 0 has read the previous candidate's warp sums
      int dummy = 0;
      const F2 lsum = warp_sum_f2(tape_pass<V, kPassLoss>(A, S, b, lane, warp, W, dummy));
      if (lane == 0) S.red_l[warp] = lsum;
      __syncthreads();
      if (threadIdx.x == 0) {
        F2 lt{0.f, 0.f};
        for (int w = 0; w < W; ++w) lt = f2_add(lt, S.red_l[w]);
        loss_out[b * K + k] = __fdiv_rn(f2_val(lt), (float)A.N);
      }
    }
    __syncthreads();  // the next problem's staging overwrites the tables
  }
}

// Rows the fit's liveness assignment needs per tape (the same events as in
// stage_problem: a row is taken at the first parent's sweep, or at the node's own
// sweep when it has no parent, and freed after the node's sweep), the batch's largest
// into stats[5].  One warp per tape, lane 0 walks the tape; tapes longer than 128
// nodes to the root count all their operator nodes (a bound).
__global__ void __launch_bounds__(256) tape_live_kernel(const uint32_t* __restrict__ desc,
                                                        const int32_t* __restrict__ meta, int64_t B, int64_t M,
                                                        int32_t* __restrict__ stats) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  int best = 0;
  for (int64_t b = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); b < B; b += warps) {
    if (lane != 0) continue;
    const int L = meta[b * 4 + 1] + 1;
    const uint32_t* d = desc + b * M;
    int live = 0;
    if (L > 128) {
      for (int k = 0; k < L; ++k) live += is_operator_node(code_of(d[k])) ? 1 : 0;
    } else {
      uint64_t held[2] = {0ull, 0ull};
      auto has = [&](int k) { return (held[k >> 6] >> (k & 63)) & 1ull; };
      auto take = [&](int k, int& cur) { held[k >> 6] |= 1ull << (k & 63); ++cur; live = cur > live ? cur : live; };
      int cur = 0;
      const int R = L - 1;
      if (is_operator_node(code_of(d[R]))) take(R, cur);
      for (int k = R; k >= 0; --k) {
        const uint32_t w = d[k];
        const int code = code_of(w);
        if (!is_operator_node(code)) continue;
        if (!has(k)) take(k, cur);
        --cur;
        const int ar = arity_of(code);
        for (int j = 0; j < ar; ++j) {
          const int c = j == 0 ? child0(w) : child1(w);
          if (is_operator_node(code_of(d[c])) && !has(c)) take(c, cur);
        }
      }
    }
    best = live > best ? live : best;
  }
  if (lane == 0 && best > 0) atomicMax(stats + 5, best);
}

static int fit_defaults(const sr_fit_options* o, sr_fit_options& r) {
  r.max_iter = 100;
  r.history_size = 10;
  r.tolerance_grad = 1e-7;
  r.line_search = 0;
  r.line_search_max_iter = 10;
  r.eps = 1e-10;
  r.objective = 0;
  r.warps_per_block = 0;
  r.points_per_lane = 0;
  r.grid_blocks = 0;
  r.max_operators = 0;
  r.max_live = 0;
  if (o) r = *o;
  if (r.max_iter < 0 || r.history_size < 1 || r.line_search < 0 || r.line_search > 1 || r.line_search_max_iter < 0 ||
      r.objective < 0 || r.objective > 1 || r.max_operators < 0 || r.max_live < 0) {
    set_error("invalid fit options");
    return SR_ERR_INVALID_ARGUMENT;
  }
  if (r.points_per_lane != 0 && r.points_per_lane != 1 && r.points_per_lane != 2 && r.points_per_lane != 4) {
    set_error("points_per_lane must be 0 (automatic), 1, 2 or 4");
    return SR_ERR_INVALID_ARGUMENT;
  }
  return SR_OK;
}

static int spl_for(int Kmax) {
  if (Kmax + 1 <= 32) return 1;
  if (Kmax + 1 <= 64) return 2;
  if (Kmax + 1 <= 128) return 4;
  return 0;
}

struct FitShape {
  int V, SPL, warps, blocks, Imax, Amax, VR;
  size_t smem;
  size_t ring_off;  // > 0: the L-BFGS history sits in shared memory from this byte offset
};


template <int V, int SPL>
static void* fit_kernel_ptr() {
  return reinterpret_cast<void*>(fit_lbfgs_kernel<V, SPL>);
}

static void* pick_kernel(int V, int SPL) {
  switch (V * 10 + SPL) {
    case 11: return fit_kernel_ptr<1, 1>();
    case 12: return fit_kernel_ptr<1, 2>();
    case 14: return fit_kernel_ptr<1, 4>();
    case 21: return fit_kernel_ptr<2, 1>();
    case 22: return fit_kernel_ptr<2, 2>();
    case 24: return fit_kernel_ptr<2, 4>();
    case 41: return fit_kernel_ptr<4, 1>();
    case 42: return fit_kernel_ptr<4, 2>();
    case 44: return fit_kernel_ptr<4, 4>();
    default: return nullptr;
  }
}

// Launch shape.  A CTA of W warps works on one problem, each warp on every W-th
// chunk of 32V points, so an expensive problem (many closures) finishes W times
// sooner and the tail of the persistent grid shrinks.  Unless the caller fixes
// them: V = 1 (two or four points per lane were slower on every workload timed on a
// GB300: README problem 115 ms at V = 2 against 79 ms at V = 1), W the smallest
// power of two that leaves at most 64 points to a warp (1..8), doubled while the
// batch alone would leave the GPU short of 16 warps per SM and a warp still gets more
// than 32 points (1024 README problems: 6.2 ms at W = 4 against 15.7 ms at W = 1).
// The warp tables hold a row per distinct variable of a tape: VR = min(n_x, Lmax) rows.
static int fit_shape(int64_t B, int64_t N, int64_t n_x, int Lmax, int Kmax, const sr_fit_options& o, FitShape& sh) {
  const int Imax = (o.max_operators > 0 && o.max_operators < Lmax) ? o.max_operators : Lmax;
  sh.Imax = Imax;
  // adjoint rows: the most operator-node adjoints live at once (rows are assigned by
  // liveness), at most one per operator node
  const int Amax = (o.max_live > 0 && o.max_live < Imax) ? o.max_live : Imax;
  sh.Amax = Amax;
  sh.VR = (int)(n_x < 1 ? 1 : (n_x < Lmax ? n_x : Lmax));
  sh.SPL = spl_for(Kmax);
  if (!sh.SPL) {
    set_error("at most 127 learnable constants per tape are supported (got %d)", Kmax);
    return SR_ERR_UNSUPPORTED;
  }
  int dev = 0, sms = 0, optin = 0;
  if (cuda_check(cudaGetDevice(&dev), "cudaGetDevice") ||
      cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count") ||
      cuda_check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "shared memory limit"))
    return SR_ERR_CUDA;
  int W = o.warps_per_block;
  if (W <= 0) {
    W = 1;
    while (W < 8 && (int64_t)W * 64 < N) W *= 2;
    const int64_t want_warps = (int64_t)(sms > 0 ? sms : 148) * 16;
    while (W < 8 && (int64_t)W * 32 < N && B * W < want_warps) W *= 2;
  }
  if (W > 8) W = 8;  // __launch_bounds__(256)
  const int vc[3] = {1, 2, 4};
  double best = -1.0;
  int bestV = 0, bestPerSm = 0;
  for (int w = W; w >= 1 && best < 0; w >>= 1) {
    for (int vi = 0; vi < 3; ++vi) {
      const int V = vc[vi];
      if (o.points_per_lane ? V != o.points_per_lane : V != 1) continue;
      void* k = pick_kernel(V, sh.SPL);
      if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, optin) != cudaSuccess) {
        set_error("fit kernel shared memory attribute failed");
        return SR_ERR_CUDA;
      }
      const size_t cb = fit_cta_bytes(Lmax, Imax, Amax, Kmax, V, w, sh.VR);
      if (cb > (size_t)optin) continue;
      int per_sm = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, w * 32, cb) != cudaSuccess || per_sm < 1)
        continue;
      const double score = (double)per_sm * w;
      if (score > best) {
        best = score;
        bestV = V;
        bestPerSm = per_sm;
        W = w;
      }
    }
    if (best < 0 && o.warps_per_block > 0) break;
  }
  if (best < 0) {
    set_error("tape of %d nodes does not fit in shared memory for the fit kernel", Lmax);
    return SR_ERR_UNSUPPORTED;
  }
  sh.V = bestV;
  sh.warps = W;
  sh.smem = fit_cta_bytes(Lmax, Imax, Amax, Kmax, bestV, W, sh.VR);
  // Warp 0 reads the L-BFGS history for every direction: keep it in shared memory
  // when that costs no resident CTA, else in the workspace.
  sh.ring_off = 0;
  {
    const size_t off = fit_align16(sh.smem), with = off + hist_block_bytes(o.history_size, sh.SPL);
    int per_sm = 0;
    if (with <= (size_t)optin &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pick_kernel(bestV, sh.SPL), W * 32, with) ==
            cudaSuccess &&
        per_sm >= bestPerSm) {
      sh.ring_off = off;
      sh.smem = with;
    }
  }
  int64_t blocks = o.grid_blocks > 0 ? o.grid_blocks : (int64_t)sms * bestPerSm;
  if (blocks > B) blocks = B;  // one problem per CTA at a time
  if (blocks < 1) blocks = 1;
  sh.blocks = (int)blocks;
  return SR_OK;
}

// Workspace of a launch: the work counter, and the L-BFGS history unless it sits in
// shared memory (rings_anyway: the size with the history, an upper bound for any n_x).
static int64_t ws_bytes_for(const FitShape& sh, int hist, bool rings_anyway = false) {
  if (sh.ring_off && !rings_anyway) return 256;
  return 256 + (int64_t)sh.blocks * (int64_t)hist_block_bytes(hist, sh.SPL);
}

}  // namespace sr

extern "C" {

int64_t sr_fit_workspace_bytes(int64_t B, int64_t N, int64_t M, int32_t max_len, int32_t max_consts,
                               const sr_fit_options* opt) {
  sr_fit_options o;
  if (sr::fit_defaults(opt, o)) return -1;
  if (max_len < 0 || max_consts < 0 || B < 0 || N < 0 || M < 0) {
    sr::set_error("negative size");
    return -1;
  }
  sr::FitShape sh;
  // the same node-table size sr_fit_lbfgs uses; one variable row gives the smallest
  // tables, hence the most resident CTAs: an upper bound for any n_x (sr_fit_lbfgs
  // shrinks its grid to the workspace it is given)
  const int Lmax = (max_len > 0 && max_len < M) ? max_len : (int)(M < 1 ? 1 : M);
  if (sr::fit_shape(B, N, 1, Lmax, max_consts, o, sh)) return -1;
  return sr::ws_bytes_for(sh, o.history_size, true);
}

int sr_tape_live_rows(const uint32_t* desc, const int32_t* meta, int64_t B, int64_t M, int32_t* stats, void* stream) {
  if (B < 0 || M < 0) { sr::set_error("negative size"); return SR_ERR_INVALID_ARGUMENT; }
  if (M > sr::kMaxNodes) { sr::set_error("tapes longer than %d nodes are not supported", sr::kMaxNodes); return SR_ERR_UNSUPPORTED; }
  if (B == 0 || M == 0) return SR_OK;
  if (!desc || !meta || !stats) { sr::set_error("null pointer argument"); return SR_ERR_INVALID_ARGUMENT; }
  int64_t blocks = (B + 7) / 8;
  if (blocks > 65535) blocks = 65535;
  sr::tape_live_kernel<<<(unsigned)blocks, 256, 0, sr::as_stream(stream)>>>(desc, meta, B, M, stats);
  return sr::launch_check("tape_live_kernel");
}

int sr_fit_launch_shape(int64_t B, int64_t N, int64_t n_x, int64_t M, int32_t max_len, int32_t max_consts,
                        const sr_fit_options* opt, int32_t* shape) {
  sr_fit_options o;
  int rc = sr::fit_defaults(opt, o);
  if (rc) return rc;
  if (!shape) { sr::set_error("null shape"); return SR_ERR_INVALID_ARGUMENT; }
  if (B < 0 || M < 0 || N < 0 || n_x < 0 || max_len < 0 || max_consts < 0) {
    sr::set_error("negative size");
    return SR_ERR_INVALID_ARGUMENT;
  }
  if (M > sr::kMaxNodes) { sr::set_error("tapes longer than %d nodes are not supported", sr::kMaxNodes); return SR_ERR_UNSUPPORTED; }
  sr::FitShape sh;
  const int Lmax = (max_len > 0 && max_len < M) ? max_len : (int)(M < 1 ? 1 : M);
  rc = sr::fit_shape(B, N, n_x, Lmax, max_consts, o, sh);
  if (rc) return rc;
  shape[0] = sh.V;
  shape[1] = sh.warps;
  shape[2] = sh.blocks;
  return SR_OK;
}

int sr_fit_screen(const float* X, int64_t N, int64_t n_x, const float* Y, const uint32_t* desc, const int32_t* meta,
                  int64_t B, int64_t M, const float* C_sets, int64_t c_sk, int64_t c_sb, int64_t c_sm, int64_t K,
                  float* loss_out, int32_t max_len, int32_t max_consts, const sr_fit_options* opt, int32_t* status,
                  void* stream) {
  using namespace sr;
  sr_fit_options o;
  int rc = fit_defaults(opt, o);
  if (rc) return rc;
  if (B < 0 || M < 0 || N < 0 || n_x < 0 || K < 0 || max_len < 0 || max_consts < 0) {
    set_error("negative size");
    return SR_ERR_INVALID_ARGUMENT;
  }
  if (M > kMaxNodes) { set_error("tapes longer than %d nodes are not supported", kMaxNodes); return SR_ERR_UNSUPPORTED; }
  if (!status) { set_error("null status"); return SR_ERR_INVALID_ARGUMENT; }
  rc = cuda_check(cudaMemsetAsync(status, 0, sizeof(int32_t), as_stream(stream)), "status reset");
  if (rc || B == 0 || M == 0 || K == 0) return rc;
  if (N == 0) { set_error("screening needs at least one data point"); return SR_ERR_INVALID_ARGUMENT; }
  if (!desc || !meta || !C_sets || !loss_out || (o.objective == 0 && !Y) || (n_x > 0 && !X)) {
    set_error("null pointer argument");
    return SR_ERR_INVALID_ARGUMENT;
  }
  FitShape sh;
  const int Lmax = (max_len > 0 && max_len < M) ? max_len : (int)M;
  rc = fit_shape(B, N, n_x, Lmax, max_consts, o, sh);
  if (rc) return rc;
  FitArgs A{};
  A.X = X; A.N = N; A.n_x = n_x; A.Y = o.objective == 0 ? Y : nullptr;
  A.desc = desc; A.meta = meta; A.B = B; A.M = M;
  A.c_sb = c_sb; A.c_sm = c_sm;
  A.objective = o.objective;
  A.Lmax = Lmax; A.Kmax = max_consts; A.Imax = sh.Imax; A.Amax = sh.Amax; A.VR = sh.VR;
  A.status = status;
  void* k = sh.V == 1 ? reinterpret_cast<void*>(fit_screen_kernel<1>)
                      : (sh.V == 2 ? reinterpret_cast<void*>(fit_screen_kernel<2>) : reinterpret_cast<void*>(fit_screen_kernel<4>));
  int dev = 0, optin = 0;
  if (cuda_check(cudaGetDevice(&dev), "cudaGetDevice") ||
      cuda_check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "shared memory limit") ||
      cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, optin), "screen smem attribute"))
    return SR_ERR_CUDA;
  const float* Cs = C_sets;
  int64_t csk = c_sk, kk = K;
  float* lo = loss_out;
  void* args[] = {&A, &Cs, &csk, &kk, &lo};
  return cuda_check(cudaLaunchKernel(k, dim3(sh.blocks), dim3(sh.warps * 32), args, sh.smem, as_stream(stream)),
                    "fit_screen_kernel");
}

int sr_fit_lbfgs(const float* X, int64_t N, int64_t n_x, const float* Y, const uint32_t* desc, const int32_t* meta,
                 int64_t B, int64_t M, const float* C_init, float* C_out, int64_t c_sb, int64_t c_sm, float* Y_final,
                 int32_t* iters_out, float* loss_out, int32_t* evals_out, const int32_t* order, int32_t max_len,
                 int32_t max_consts, const sr_fit_options* opt, void* workspace, int64_t workspace_bytes, int32_t* status,
                 void* stream) {
  using namespace sr;
  sr_fit_options o;
  int rc = fit_defaults(opt, o);
  if (rc) return rc;
  if (B < 0 || M < 0 || N < 0 || n_x < 0 || max_len < 0 || max_consts < 0) {
    set_error("negative size");
    return SR_ERR_INVALID_ARGUMENT;
  }
  if (M > kMaxNodes) { set_error("tapes longer than %d nodes are not supported", kMaxNodes); return SR_ERR_UNSUPPORTED; }
  if (!status) { set_error("null status"); return SR_ERR_INVALID_ARGUMENT; }
  cudaStream_t st = as_stream(stream);
  rc = cuda_check(cudaMemsetAsync(status, 0, sizeof(int32_t), st), "status reset");
  if (rc || B == 0 || M == 0) return rc;
  if (N == 0) { set_error("optimize needs at least one data point"); return SR_ERR_INVALID_ARGUMENT; }
  if (!desc || !meta || !C_init || !C_out || (o.objective == 0 && !Y) || (n_x > 0 && !X) || !workspace) {
    set_error("null pointer argument");
    return SR_ERR_INVALID_ARGUMENT;
  }
  FitShape sh;
  const int Lmax = (max_len > 0 && max_len < M) ? max_len : (int)M;
  rc = fit_shape(B, N, n_x, Lmax, max_consts, o, sh);
  if (rc) return rc;
  // fewer persistent CTAs only lengthen each one's share of the queue
  while (sh.blocks > 1 && ws_bytes_for(sh, o.history_size) > workspace_bytes)
    sh.blocks = sh.blocks > 8 ? sh.blocks * 3 / 4 : sh.blocks - 1;
  const int64_t need = ws_bytes_for(sh, o.history_size);
  if (workspace_bytes < need) {
    set_error("workspace too small: %lld < %lld bytes", (long long)workspace_bytes, (long long)need);
    return SR_ERR_WORKSPACE;
  }
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  FitArgs A;
  A.X = X; A.N = N; A.n_x = n_x; A.Y = o.objective == 0 ? Y : nullptr;
  A.desc = desc; A.meta = meta; A.B = B; A.M = M;
  A.C_init = C_init; A.C_out = C_out; A.c_sb = c_sb; A.c_sm = c_sm;
  A.Y_final = Y_final; A.iters_out = iters_out; A.loss_out = loss_out; A.evals_out = evals_out;
  A.order = order;
  A.max_iter = o.max_iter; A.hist = o.history_size; A.ls_kind = o.line_search; A.ls_max = o.line_search_max_iter;
  A.objective = o.objective; A.tol = o.tolerance_grad; A.eps = o.eps;
  A.Lmax = Lmax; A.Kmax = max_consts; A.Imax = sh.Imax; A.Amax = sh.Amax; A.VR = sh.VR;
  A.counter = reinterpret_cast<int*>(ws);
  A.ws_hist = sh.ring_off ? nullptr : ws + 256;
  A.ring_off = (int)sh.ring_off;
  A.status = status;
  rc = cuda_check(cudaMemsetAsync(ws, 0, 256, st), "work counter reset");
  if (rc) return rc;
  void* k = pick_kernel(sh.V, sh.SPL);
  void* args[] = {&A};
  rc = cuda_check(cudaLaunchKernel(k, dim3(sh.blocks), dim3(sh.warps * 32), args, sh.smem, st), "fit_lbfgs_kernel");
  return rc;
}

}  // extern "C"

// ---------------------------------------------------------------------------------
// Fit without any device allocation by the caller.
//
// Some callers cannot hand this library a workspace: a host process whose device
// memory is owned entirely by its own pool allocator and which forbids any other
// cudaMalloc (cudaMalloc synchronises the device and may fail under the pool's
// budget), or a latency-bound service that must not allocate on its request path.
// For them the fit's scratch (work counter, per-CTA L-BFGS history) lives in
// a file-scope device array of fixed size instead of a caller buffer.
// ---------------------------------------------------------------------------------
namespace sr {

constexpr int64_t kStaticFitScratchBytes = 16LL << 20;  // 16 MiB, held on every device that loads the library
static __device__ __align__(256) unsigned char g_fit_static_scratch[kStaticFitScratchBytes];

// Device address of g_fit_static_scratch on the current device (the name is only a
// host-side stand-in in host code).  Looked up on every call: the lookup allocates
// nothing and does not synchronise, and an address kept from an earlier call would
// dangle after a device reset.
static int static_scratch_address(void** out) {
  void* p = nullptr;
  const int rc = cuda_check(cudaGetSymbolAddress(&p, g_fit_static_scratch), "cudaGetSymbolAddress(static fit scratch)");
  if (rc) return rc;
  *out = p;
  return SR_OK;
}

}  // namespace sr

extern "C" int sr_fit_lbfgs_static_scratch(const float* X, int64_t N, int64_t n_x, const float* Y,
                                           const uint32_t* desc, const int32_t* meta, int64_t B, int64_t M,
                                           const float* C_init, float* C_out, int64_t c_sb, int64_t c_sm,
                                           float* Y_final, int32_t* iters_out, float* loss_out, int32_t* evals_out,
                                           const int32_t* order, int32_t max_len, int32_t max_consts,
                                           const sr_fit_options* opt, int32_t* status, void* stream) {
  using namespace sr;
  sr_fit_options o;
  int rc = fit_defaults(opt, o);
  if (rc) return rc;
  if (B < 0 || M < 0 || max_len < 0 || max_consts < 0) { set_error("negative size"); return SR_ERR_INVALID_ARGUMENT; }
  if (B == 0 || M == 0) return sr_fit_lbfgs(X, N, n_x, Y, desc, meta, B, M, C_init, C_out, c_sb, c_sm, Y_final,
                                            iters_out, loss_out, evals_out, order, max_len, max_consts, &o, nullptr,
                                            0, status, stream);
  // Persistent grid: fewer CTAs only lengthen the work queue per warp, so shrink the
  // grid until its L-BFGS history fits in the static array.
  FitShape sh;
  const int Lmax = (max_len > 0 && max_len < M) ? max_len : (int)M;
  rc = fit_shape(B, N, n_x, Lmax, max_consts, o, sh);
  if (rc) return rc;
  int64_t blocks = sh.blocks;
  while (blocks >= 1) {
    FitShape t = sh;
    t.blocks = (int)blocks;
    if (ws_bytes_for(t, o.history_size) <= kStaticFitScratchBytes) break;
    blocks = blocks > 8 ? blocks * 3 / 4 : blocks - 1;
  }
  if (blocks < 1) {
    FitShape t = sh;
    t.blocks = 1;
    set_error("static fit scratch is %lld bytes; one CTA of %d warps needs %lld (history_size=%d, up to %d constants); "
              "use sr_fit_lbfgs with a caller workspace",
              (long long)kStaticFitScratchBytes, sh.warps, (long long)ws_bytes_for(t, o.history_size), o.history_size,
              max_consts);
    return SR_ERR_WORKSPACE;
  }
  void* scratch = nullptr;
  rc = static_scratch_address(&scratch);
  if (rc) return rc;
  o.grid_blocks = (int32_t)blocks;
  o.warps_per_block = sh.warps;
  o.points_per_lane = sh.V;
  return sr_fit_lbfgs(X, N, n_x, Y, desc, meta, B, M, C_init, C_out, c_sb, c_sm, Y_final, iters_out, loss_out,
                      evals_out, order, max_len, max_consts, &o, scratch, kStaticFitScratchBytes, status, stream);
}
