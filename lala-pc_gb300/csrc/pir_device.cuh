// Device-side PIR propagators for sm_103a.
//
// One propagator application follows lala-pc's PIR::deduce(bytecode_type)
// (include/lala/pir.hpp:721-817) and its helpers (:407-718): the same
// per-opcode update order (later bounds read the already-updated earlier ones),
// the same +-inf guards, the same early-outs.  Bounds are int32; an
// intermediate that would leave int32 saturates to INT32_MIN/INT32_MAX
// (add.sat/sub.sat, or exact int64 then clamp), which is monotone and therefore
// keeps the fixpoint independent of the propagation order.
//
// The store is abstracted by a policy `S` with
//   Itv  load(int v)                         -- current interval of v
//   int  embed(int v, Itv seen, Itv r, int&) -- meet r into v; `seen` is the
//        value load() returned for v; returns the number of bounds narrowed
//        and sets the failure flag when v becomes empty.
// GlobalStore (HBM, device-scope atomics), SmemStore (shared memory, block
// atomics) and LocalStore (a thread-private store) implement it.
#pragma once
#include <climits>
#include <cstdint>

namespace pirgpu {

enum : int {
  OP_ADD = 0, OP_MUL = 1, OP_TDIV = 2, OP_FDIV = 3, OP_CDIV = 4, OP_EDIV = 5,
  OP_MIN = 6, OP_MAX = 7, OP_EQ = 8, OP_LEQ = 9, OP_COUNT = 10,
  OP_NOP = 15  // padding slot of the bytecode arrays
};

constexpr int INF = INT_MAX;   // pir.hpp:403
constexpr int MINF = INT_MIN;  // pir.hpp:404

struct Itv {
  int l, u;
};

static __host__ __device__ __forceinline__ Itv mk(int l, int u) { Itv r; r.l = l; r.u = u; return r; }

// Empty interval: lb > ub, or a bound at its bottom sentinel (ZLB bot = +inf,
// ZUB bot = -inf).
static __device__ __forceinline__ bool is_bot(Itv a) { return a.l > a.u || a.l == INF || a.u == MINF; }
static __device__ __forceinline__ bool eq(Itv a, int l, int u) { return a.l == l && a.u == u; }

static __device__ __forceinline__ int sadd(int a, int b) {
  int r;
  asm("add.sat.s32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
static __device__ __forceinline__ int ssub(int a, int b) {
  int r;
  asm("sub.sat.s32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
static __device__ __forceinline__ int sneg(int a) { return ssub(0, a); }
static __device__ __forceinline__ int cl(long long v) {
  return (int)(v > (long long)INF ? (long long)INF : (v < (long long)MINF ? (long long)MINF : v));
}
static __device__ __forceinline__ long long mn(long long a, long long b) { return a < b ? a : b; }
static __device__ __forceinline__ long long mx(long long a, long long b) { return a > b ? a : b; }

// Truncating quotient and remainder, b != 0: 32-bit division when both
// operands fit in int32 (and the quotient does), the 64-bit routine otherwise.
static __device__ __forceinline__ void d_qr(long long a, long long b, long long &q, long long &r) {
  if (a >= INT_MIN && a <= INT_MAX && b >= INT_MIN && b <= INT_MAX && !(a == INT_MIN && b == -1)) {
    const int qi = (int)a / (int)b;
    q = qi;
    r = a - (long long)qi * b;
  } else {
    q = a / b;
    r = a - q * b;
  }
}
// Integer divisions by their definitions (cuda-battery tdiv/fdiv/cdiv/ediv), b != 0.
static __device__ __forceinline__ long long d_fdiv(long long a, long long b) {
  long long q, r;
  d_qr(a, b, q, r);
  return (r != 0 && ((r ^ b) < 0)) ? q - 1 : q;
}
static __device__ __forceinline__ long long d_cdiv(long long a, long long b) {
  long long q, r;
  d_qr(a, b, q, r);
  return (r != 0 && ((r ^ b) >= 0)) ? q + 1 : q;
}
static __device__ __forceinline__ long long d_ediv(long long a, long long b) {
  long long q, r;
  d_qr(a, b, q, r);
  return r < 0 ? (b > 0 ? q - 1 : q + 1) : q;
}
static __device__ __forceinline__ long long d_tdiv(long long a, long long b) {
  long long q, r;
  d_qr(a, b, q, r);
  return q;
}
static __device__ __forceinline__ long long d_div(int op, long long a, long long b) {
  switch (op) {
    case OP_TDIV: return d_tdiv(a, b);
    case OP_CDIV: return d_cdiv(a, b);
    case OP_FDIV: return d_fdiv(a, b);
    default: return d_ediv(a, b);
  }
}
// 32-bit truncating quotient and remainder; floor/ceil follow from the sign of r.
static __device__ __forceinline__ void qr32(int a, int b, int &q, int &r) {
  q = a / b;
  r = a - q * b;
}

// ---------------------------------------------------------------- MUL -------
// y = x / z for x = y * z (pir.hpp:702-718).  r1 = x, r2 = the factor being
// narrowed, r3 = the other factor.
static __device__ __forceinline__ void mul_inv(const Itv &r1, Itv &r2, Itv &r3) {
  const bool xnz = (r1.l > 0) | (r1.u < 0);
  if (xnz) {
    if (r3.l == 0) r3.l = 1;
    if (r3.u == 0) r3.u = -1;
  }
  if (xnz && r3.l < 0 && r3.u > 0) {
    r2.l = max(r2.l, min(r1.l, r1.u == MINF ? INF : sneg(r1.u)));
    r2.u = min(r2.u, max(r1.l == INF ? MINF : sneg(r1.l), r1.u));
  } else if (xnz | (r3.l > 0) | (r3.u < 0)) {
    if (r1.l == MINF || r1.u == INF || r3.l == MINF || r3.u == INF) return;
    if (is_bot(r3)) return;
    // The reference takes the min of cdiv and the max of fdiv over the four
    // corners (x_i, z_j).  Here z is sign-definite (z > 0 or z < 0 after the
    // zero endpoints were moved), so a / b is monotone in each argument over
    // the box and its extremes sit at corners a sign analysis names; ceil and
    // floor are monotone, so cdiv / fdiv at those corners are the corner
    // minimum / maximum: two divisions instead of eight.  (An empty x gives
    // other values than the corner search, but then the failure is already
    // flagged and the bounds are not used.)  r1.l > MINF here, so no quotient
    // overflows int32.
    const bool zpos = r3.l > 0;
    int al, bl, au, bu;  // min a/b at (al, bl), max a/b at (au, bu)
    if (zpos) {
      al = r1.l;
      bl = r1.l >= 0 ? r3.u : r3.l;
      au = r1.u;
      bu = r1.u >= 0 ? r3.l : r3.u;
    } else {
      al = r1.u;
      bl = r1.u >= 0 ? r3.u : r3.l;
      au = r1.l;
      bu = r1.l >= 0 ? r3.l : r3.u;
    }
    // A bound moves only when the quotient passes it: cdiv(a, b) > n iff
    // a / b > n iff a > n * b (b > 0) or a < n * b (b < 0), and
    // fdiv(a, b) < n iff a < n * b (b > 0) or a > n * b (b < 0) -- one exact
    // 64-bit product instead of a division when nothing would change.
    const long long nl = (long long)r2.l * bl, nu = (long long)r2.u * bu;
    if (bl > 0 ? (long long)al > nl : (long long)al < nl) {
      int q, m;
      qr32(al, bl, q, m);
      // cdiv = q + (r != 0 && sign(r) == sign(b))
      r2.l = max(r2.l, q + ((m != 0) & ((m ^ bl) >= 0)));
    }
    if (bu > 0 ? (long long)au < nu : (long long)au > nu) {
      int q, m;
      qr32(au, bu, q, m);
      // fdiv = q - (r != 0 && sign(r) != sign(b))
      r2.u = min(r2.u, q - ((m != 0) & ((m ^ bu) < 0)));
    }
  }
}

// ----------------------------------------------------------- divisions ------
// Interval helpers of the division propagators.  Hull (join) treats the empty
// interval as neutral.
static __device__ __forceinline__ Itv top() { return mk(MINF, INF); }
static __device__ __forceinline__ Itv bot() { return mk(INF, MINF); }
static __device__ __forceinline__ Itv of64(long long l, long long u) { return mk(cl(l), cl(u)); }
static __device__ __forceinline__ Itv hull(Itv a, Itv b) {
  if (is_bot(b)) return a;
  if (is_bot(a)) return b;
  return mk(min(a.l, b.l), max(a.u, b.u));
}
static __device__ __forceinline__ void meet(Itv &a, Itv b) {
  a.l = max(a.l, b.l);
  a.u = min(a.u, b.u);
}

// r1 = r2 / r3 forward (pir.hpp:449-467)
static __device__ __forceinline__ void itv_div(int op, Itv &r1, Itv &r2, Itv &r3) {
  if (r3.l < 0 && r3.u > 0) {
    r1.l = max(r1.l, min(r2.l, r2.u == MINF ? INF : sneg(r2.u)));
    r1.u = min(r1.u, max(r2.l == INF ? MINF : sneg(r2.l), r2.u));
  } else {
    if (r3.l == 0) r3.l = 1;
    if (r3.u == 0) r3.u = -1;
    if (r2.l == MINF || r2.u == INF || r3.l == MINF || r3.u == INF) return;
    if (is_bot(r3)) return;
    // The reference's min / max over the four corners: z is sign-definite
    // here and every one of the four divisions is monotone in y / z, so the
    // extremes are at the corners a sign analysis names (as in mul_inv).
    long long lo, hi;
    if (r3.l > 0) {
      lo = d_div(op, r2.l, r2.l >= 0 ? r3.u : r3.l);
      hi = d_div(op, r2.u, r2.u >= 0 ? r3.l : r3.u);
    } else {
      lo = d_div(op, r2.u, r2.u >= 0 ? r3.u : r3.l);
      hi = d_div(op, r2.l, r2.l >= 0 ? r3.l : r3.u);
    }
    r1.l = cl(mx(r1.l, lo));
    r1.u = cl(mn(r1.u, hi));
  }
}

// Numerator bounds y for x = fdiv(y, z) (pir.hpp:469-479); x = r1, z = r3.
static __device__ Itv num_fdiv(Itv r1, Itv r3) {
  const long long xl = r1.l, xu = r1.u, zl = r3.l, zu = r3.u;
  if (zl < 0 && zu > 0)
    return of64(mn(mn(xl, -xu), mn(xl * zu, (xu + 1) * zl + 1)),
                mx(mx(-xl, xu), mx(xl * zl, (xu + 1) * zu - 1)));
  if (zl > 0 || zu < 0)
    return of64(mn(mn(xl * zl, xl * zu), mn((xu + 1) * zl + 1, (xu + 1) * zu + 1)),
                mx(mx(xl * zl, xl * zu), mx((xu + 1) * zl - 1, (xu + 1) * zu - 1)));
  return top();
}
// pir.hpp:481-491
static __device__ Itv num_cdiv(Itv r1, Itv r3) {
  const long long xl = r1.l, xu = r1.u, zl = r3.l, zu = r3.u;
  if (zl < 0 && zu > 0)
    return of64(mn(mn(xl, -xu), mn(xu * zl, (xl - 1) * zu + 1)),
                mx(mx(-xl, xu), mx(xu * zu, (xl - 1) * zl - 1)));
  if (zl > 0 || zu < 0)
    return of64(mn(mn(xu * zl, xu * zu), mn((xl - 1) * zl + 1, (xl - 1) * zu + 1)),
                mx(mx(xu * zl, xu * zu), mx((xl - 1) * zl - 1, (xl - 1) * zu - 1)));
  return top();
}
// pir.hpp:493-507
static __device__ Itv num_tdiv(Itv r1, Itv r3) {
  if (r1.l > 0) return num_fdiv(r1, r3);
  if (r1.u < 0) return num_cdiv(r1, r3);
  if (r1.l <= 0 && 0 <= r1.u) {
    const long long zl = r3.l, zu = r3.u;
    Itv r = of64(mn(zl, -zu) + 1, mx(-zl, zu) - 1);
    if (r1.l != 0) r = hull(r, num_cdiv(mk(r1.l, -1), r3));
    if (r1.u != 0) r = hull(r, num_fdiv(mk(1, r1.u), r3));
    return r;
  }
  return top();
}
// pir.hpp:510-517
static __device__ Itv num_ediv(Itv r1, Itv r3) {
  if (r3.l > 0) return num_fdiv(r1, r3);
  if (r3.u < 0) return num_cdiv(r1, r3);
  if (r3.l < 0 && r3.u > 0) return hull(num_cdiv(r1, mk(r3.l, -1)), num_fdiv(r1, mk(1, r3.u)));
  return top();
}

// Divisor bounds z for x = fdiv(y, z) when x <= -2 or x >= 1 and y has a sign
// (the direct cases of pir.hpp:522-534).
static __device__ Itv den_fdiv_signed(long long xl, long long xu, long long yl, long long yu) {
  if (yl > 0)
    return of64(mn(d_fdiv(yl, xu + 1), d_fdiv(yu, xu + 1)) + 1, mx(d_fdiv(yl, xl), d_fdiv(yu, xl)));
  return of64(mn(d_cdiv(yl, xl), d_cdiv(yu, xl)), mx(d_cdiv(yl, xu + 1), d_cdiv(yu, xu + 1)) - 1);
}
// pir.hpp:522-547: x <= -2 or x >= 1, any y.
static __device__ Itv den_fdiv_a(Itv r1, Itv r2) {
  const long long xl = r1.l, xu = r1.u, yl = r2.l, yu = r2.u;
  if (yl > 0 || yu < 0) return den_fdiv_signed(xl, xu, yl, yu);
  if (0 == yl && yl < yu) return den_fdiv_signed(xl, xu, 1, yu);
  if (yl < yu && yu == 0) return den_fdiv_signed(xl, xu, yl, -1);
  if (yl < 0 && 0 < yu) return hull(den_fdiv_signed(xl, xu, yl, -1), den_fdiv_signed(xl, xu, 1, yu));
  if (yl == 0 && yu == 0) return bot();
  return top();
}
// pir.hpp:548-552: x = [0, 0].
static __device__ Itv den_fdiv_zero(Itv r2) {
  if (r2.l > 0) return of64((long long)r2.l + 1, INF);
  if (r2.u < 0) return of64(MINF, (long long)r2.u - 1);
  return top();
}
// pir.hpp:553-559: x = [-1, -1].
static __device__ Itv den_fdiv_m1(Itv r2) {
  const long long yl = r2.l, yu = r2.u;
  if (yl > 0) return of64(MINF, -yl);
  if (yu < 0) return of64(-yu, INF);
  if (0 == yl && yl < yu) return mk(MINF, -1);
  if (yl < yu && yu == 0) return mk(1, INF);
  if (yl == 0 && yu == 0) return bot();
  return top();
}
// Lemma A.11, pir.hpp:520-574, with the recursion unfolded into the cases above.
static __device__ Itv den_fdiv(Itv r1, Itv r2) {
  const long long xl = r1.l, xu = r1.u;
  if (xl > 0 || xu + 1 < 0) return den_fdiv_a(r1, r2);
  if (xl == 0 && xu == 0) return den_fdiv_zero(r2);
  if (xl == -1 && xu == -1) return den_fdiv_m1(r2);
  if (xl == 0 && 0 < xu) return hull(den_fdiv_zero(r2), den_fdiv_a(mk(1, r1.u), r2));
  if (xl < -1 && xu == -1) return hull(den_fdiv_a(mk(r1.l, -2), r2), den_fdiv_m1(r2));
  if (xl <= -1 && xu >= 0) {
    Itv r = hull(den_fdiv_m1(r2), den_fdiv_zero(r2));
    if (xl != -1) r = hull(r, den_fdiv_a(mk(r1.l, -2), r2));
    if (xu != 0) r = hull(r, den_fdiv_a(mk(1, r1.u), r2));
    return r;
  }
  return top();
}

// Direct cases of den_cdiv (pir.hpp:579-591): x >= 2 or x <= -1, y signed.
static __device__ Itv den_cdiv_signed(long long xl, long long xu, long long yl, long long yu) {
  if (yl > 0)
    return of64(mn(d_cdiv(yl, xu), d_cdiv(yu, xu)), mx(d_cdiv(yl, xl - 1), d_cdiv(yu, xl - 1)) - 1);
  return of64(mn(d_fdiv(yl, xl - 1), d_fdiv(yu, xl - 1)) + 1, mx(d_fdiv(yl, xu), d_fdiv(yu, xu)));
}
// pir.hpp:579-604
static __device__ Itv den_cdiv_a(Itv r1, Itv r2) {
  const long long xl = r1.l, xu = r1.u, yl = r2.l, yu = r2.u;
  if (yl > 0 || yu < 0) return den_cdiv_signed(xl, xu, yl, yu);
  if (0 == yl && yl < yu) return den_cdiv_signed(xl, xu, 1, yu);
  if (yl < yu && yu == 0) return den_cdiv_signed(xl, xu, yl, -1);
  if (yl < 0 && 0 < yu) return hull(den_cdiv_signed(xl, xu, yl, -1), den_cdiv_signed(xl, xu, 1, yu));
  if (yl == 0 && yu == 0) return bot();
  return top();
}
// pir.hpp:605-608: x = [0, 0].
static __device__ Itv den_cdiv_zero(Itv r2) {
  if (r2.l > 0) return of64(MINF, -(long long)r2.l - 1);
  if (r2.u < 0) return of64(-(long long)r2.u + 1, INF);
  return top();
}
// pir.hpp:609-615: x = [1, 1].
static __device__ Itv den_cdiv_one(Itv r2) {
  const int yl = r2.l, yu = r2.u;
  if (yl > 0) return mk(yl, INF);
  if (yu < 0) return mk(MINF, yu);
  if (0 == yl && yl < yu) return mk(1, INF);
  if (yl < yu && yu == 0) return mk(MINF, -1);
  if (yl == 0 && yu == 0) return bot();
  return top();
}
// Lemma C.12, pir.hpp:577-630, recursion unfolded.
static __device__ Itv den_cdiv(Itv r1, Itv r2) {
  const long long xl = r1.l, xu = r1.u;
  if (xl - 1 > 0 || xu < 0) return den_cdiv_a(r1, r2);
  if (xl == 0 && xu == 0) return den_cdiv_zero(r2);
  if (xl == 1 && xu == 1) return den_cdiv_one(r2);
  if (xl < 0 && xu == 0) return hull(den_cdiv_a(mk(r1.l, -1), r2), den_cdiv_zero(r2));
  if (xl == 1 && 1 < xu) return hull(den_cdiv_one(r2), den_cdiv_a(mk(2, r1.u), r2));
  if (xl <= 0 && xu >= 1) {
    Itv r = hull(den_cdiv_one(r2), den_cdiv_zero(r2));
    if (xl != 0) r = hull(r, den_cdiv_a(mk(r1.l, -1), r2));
    if (xu != 1) r = hull(r, den_cdiv_a(mk(2, r1.u), r2));
    return r;
  }
  return top();
}

// Lemma C.13, pir.hpp:633-649.
static __device__ Itv den_tdiv_zero(Itv r2, Itv r3) {
  const long long yl = r2.l, yu = r2.u, zl = r3.l, zu = r3.u;
  if (yl > 0 && zl > 0) return of64(yl + 1, INF);
  if (yl > 0 && zu < 0) return of64(MINF, -yl - 1);
  if (yu < 0 && zl > 0) return of64(-yu + 1, INF);
  if (yu < 0 && zu < 0) return of64(MINF, yu - 1);
  return top();
}
static __device__ Itv den_tdiv(Itv r1, Itv r2, Itv r3) {
  if (r1.l > 0) return den_fdiv(r1, r2);
  if (r1.u < 0) return den_cdiv(r1, r2);
  if (r1.l == 0 && r1.u == 0) return den_tdiv_zero(r2, r3);
  if (r1.l <= 0 && 0 <= r1.u) {
    Itv r = den_tdiv_zero(r2, r3);
    if (r1.l != 0) r = hull(r, den_cdiv(mk(r1.l, -1), r2));
    if (r1.u != 0) r = hull(r, den_fdiv(mk(1, r1.u), r2));
    return r;
  }
  return top();
}
// pir.hpp:651-658
static __device__ Itv den_ediv(Itv r1, Itv r2, Itv r3) {
  if (r3.l > 0) return den_fdiv(r1, r2);
  if (r3.u < 0) return den_cdiv(r1, r2);
  if (r3.l < 0 && 0 < r3.u) return hull(den_fdiv(r1, r2), den_cdiv(r1, r2));
  return top();
}

// The three intervals of one propagator, passed to and returned from the out
// of line division code by value: a reference would take the caller's
// intervals' address and put them in local memory for every opcode.
struct Itv3 {
  Itv a, b, c;
};

// The four division opcodes (pir.hpp:780-792), out of line so that the common
// opcodes keep a small register footprint.
static __device__ __noinline__ Itv3 deduce_div(int op, Itv3 t) {
  Itv r1 = t.a, r2 = t.b, r3 = t.c;
  itv_div(op, r1, r2, r3);
  if (!is_bot(r1) && !is_bot(r3)) {
    switch (op) {
      case OP_FDIV: meet(r2, num_fdiv(r1, r3)); break;
      case OP_CDIV: meet(r2, num_cdiv(r1, r3)); break;
      case OP_TDIV: meet(r2, num_tdiv(r1, r3)); break;
      default: meet(r2, num_ediv(r1, r3)); break;
    }
    if (!is_bot(r2)) {
      switch (op) {
        case OP_FDIV: meet(r3, den_fdiv(r1, r2)); break;
        case OP_CDIV: meet(r3, den_cdiv(r1, r2)); break;
        case OP_TDIV: meet(r3, den_tdiv(r1, r2, r3)); break;
        default: meet(r3, den_ediv(r1, r2, r3)); break;
      }
    }
  }
  Itv3 out;
  out.a = r1;
  out.b = r2;
  out.c = r3;
  return out;
}

// ---------------------------------------------------------------- deduce ----
// One propagator x = y <op> z (pir.hpp:721-817) given the intervals o1, o2, o3
// read for x, y, z.  Returns the number of bounds narrowed in the store; sets
// `failed` when an empty interval is read or produced.
template <class S>
static __device__ __forceinline__ int deduce_loaded(int op, int X, int Y, int Z, const Itv o1, const Itv o2,
                                             const Itv o3, S &st, int &failed) {
  if (op == OP_NOP) return 0;
  if (is_bot(o1) || is_bot(o2) || is_bot(o3)) {
    failed = 1;
    return 0;
  }
  Itv r1 = o1, r2 = o2, r3 = o3;
  switch (op) {
    case OP_EQ: {  // pir.hpp:730-744
      if (eq(r1, 1, 1)) {
        return st.embed(Y, o2, r3, failed) + st.embed(Z, o3, r2, failed);
      } else if (eq(r1, 0, 0) && (r2.l == r2.u || r3.l == r3.u)) {
        const Itv d = mk(r2.l == r3.l ? sadd(r2.l, 1) : MINF, r2.u == r3.u ? ssub(r2.u, 1) : INF);
        return r3.l == r3.u ? st.embed(Y, o2, d, failed) : st.embed(Z, o3, d, failed);
      } else if (r2.u == r3.l && r2.l == r3.u) {
        return st.embed(X, o1, mk(1, 1), failed);
      } else if (r2.l > r3.u || r2.u < r3.l) {
        return st.embed(X, o1, mk(0, 0), failed);
      }
      return 0;
    }
    case OP_LEQ: {  // pir.hpp:745-757
      if (eq(r1, 1, 1)) {
        const Itv d = mk(r2.l, r3.u);
        return st.embed(Y, o2, d, failed) + st.embed(Z, o3, d, failed);
      } else if (eq(r1, 0, 0)) {
        return st.embed(Y, o2, mk(sadd(r3.l, 1), r2.u), failed) +
               st.embed(Z, o3, mk(r3.l, ssub(r2.u, 1)), failed);
      } else if (r2.u <= r3.l) {
        return st.embed(X, o1, mk(1, 1), failed);
      } else if (r2.l > r3.u) {
        return st.embed(X, o1, mk(0, 0), failed);
      }
      return 0;
    }
    case OP_ADD: {  // pir.hpp:758-766
      if (r2.l != MINF && r3.l != MINF) r1.l = max(r1.l, sadd(r2.l, r3.l));
      if (r2.u != INF && r3.u != INF) r1.u = min(r1.u, sadd(r2.u, r3.u));
      if (r1.l != MINF && r3.u != INF) r2.l = max(r2.l, ssub(r1.l, r3.u));
      if (r1.u != INF && r3.l != MINF) r2.u = min(r2.u, ssub(r1.u, r3.l));
      if (r1.l != MINF && r2.u != INF) r3.l = max(r3.l, ssub(r1.l, r2.u));
      if (r1.u != INF && r2.l != MINF) r3.u = min(r3.u, ssub(r1.u, r2.l));
      break;
    }
    case OP_MUL: {  // pir.hpp:767-779
      if (r2.l != MINF && r2.u != INF && r3.l != MINF && r3.u != INF) {
        const long long t1 = (long long)r2.l * r3.l, t2 = (long long)r2.l * r3.u;
        const long long t3 = (long long)r2.u * r3.l, t4 = (long long)r2.u * r3.u;
        r1.l = cl(mx(r1.l, mn(mn(t1, t2), mn(t3, t4))));
        r1.u = cl(mn(r1.u, mx(mx(t1, t2), mx(t3, t4))));
      }
      mul_inv(r1, r2, r3);
      mul_inv(r1, r3, r2);
      break;
    }
    case OP_MIN: {  // pir.hpp:793-801
      r1.l = max(r1.l, min(r2.l, r3.l));
      r1.u = min(r1.u, min(r2.u, r3.u));
      r2.l = max(r2.l, r1.l);
      if (r1.u < r3.l) r2.u = min(r2.u, r1.u);
      r3.l = max(r3.l, r1.l);
      if (r1.u < r2.l) r3.u = min(r3.u, r1.u);
      break;
    }
    case OP_MAX: {  // pir.hpp:802-810
      r1.l = max(r1.l, max(r2.l, r3.l));
      r1.u = min(r1.u, max(r2.u, r3.u));
      r2.u = min(r2.u, r1.u);
      if (r1.l > r3.u) r2.l = max(r2.l, r1.l);
      r3.u = min(r3.u, r1.u);
      if (r1.l > r2.u) r3.l = max(r3.l, r1.l);
      break;
    }
    case OP_TDIV:
    case OP_FDIV:
    case OP_CDIV:
    case OP_EDIV: {
      Itv3 t;
      t.a = r1;
      t.b = r2;
      t.c = r3;
      t = deduce_div(op, t);
      r1 = t.a;
      r2 = t.b;
      r3 = t.c;
      break;
    }
    default:
      return 0;
  }
  // pir.hpp:813-815
  return st.embed(X, o1, r1, failed) + st.embed(Y, o2, r2, failed) + st.embed(Z, o3, r3, failed);
}

// One propagator read from the store and applied (pir.hpp:387-390).
template <class S>
static __device__ __forceinline__ int deduce(int op, int X, int Y, int Z, S &st, int &failed) {
  if (op == OP_NOP) return 0;
  const Itv o1 = st.load(X), o2 = st.load(Y), o3 = st.load(Z);
  return deduce_loaded(op, X, Y, Z, o1, o2, o3, st, failed);
}

// Entailment of one propagator (pir.hpp:417-438).
static __device__ __forceinline__ bool ask(int op, Itv r1, Itv r2, Itv r3) {
  const long long xl = r1.l, xu = r1.u, yl = r2.l, yu = r2.u, zl = r3.l, zu = r3.u;
  switch (op) {
    case OP_EQ: return (xl == 1 && yu == zl && yl == zu) || (xu == 0 && (yu < zl || yl > zu));
    case OP_LEQ: return (xl == 1 && yu <= zl) || (xu == 0 && yl > zu);
    case OP_ADD: return xl == xu && yl == yu && zl == zu && xl == yl + zl;
    case OP_MUL:
      return xl == xu && ((yl == yu && zl == zu && xl == yl * zl) ||
                          (xl == 0 && ((yl == 0 && yu == 0) || (zl == 0 && zu == 0))));
    case OP_TDIV:
    case OP_CDIV:
    case OP_FDIV:
    case OP_EDIV:
      return (xl == xu && yl == yu && zl == zu && zl != 0 && xl == d_div(op, yl, zl)) ||
             (xl == yu && xu == yl && xl == 0 && (zl > 0 || zu < 0));
    case OP_MIN: return (xl == yu && xu == yl && yu <= zl) || (xl == zu && xu == zl && zu <= yl);
    case OP_MAX: return (xl == yu && xu == yl && yl >= zu) || (xl == zu && xu == zl && zl >= yu);
    default: return true;
  }
}

// ------------------------------------------------------------ stores --------
// The interval store in HBM: one int2 {lb, ub} per variable.  Loads bypass L1
// (ld.global.cg) so that bounds joined by other SMs are seen in later rounds;
// joins are device-scope atomicMax / atomicMin, issued only when the new bound
// is tighter than the one read.
struct GlobalStore {
  int2 *s;
  __device__ __forceinline__ Itv load(int v) const {
    const int2 t = __ldcg(s + v);
    return mk(t.x, t.y);
  }
  __device__ __forceinline__ int embed(int v, Itv seen, Itv r, int &failed) const {
    int n = 0, nl = seen.l, nu = seen.u;
    if (r.l > seen.l) {
      const int old = atomicMax(&s[v].x, r.l);
      n += old < r.l;
      nl = max(old, r.l);
    }
    if (r.u < seen.u) {
      const int old = atomicMin(&s[v].y, r.u);
      n += old > r.u;
      nu = min(old, r.u);
    }
    if (n && is_bot(mk(nl, nu))) failed = 1;
    return n;
  }
};

// A store staged in shared memory (an instance that fits on one SM).
struct SmemStore {
  int2 *s;
  __device__ __forceinline__ Itv load(int v) const {
    const volatile int2 *p = s + v;
    return mk(p->x, p->y);
  }
  __device__ __forceinline__ int embed(int v, Itv seen, Itv r, int &failed) const {
    int n = 0, nl = seen.l, nu = seen.u;
    if (r.l > seen.l) {
      const int old = atomicMax(&s[v].x, r.l);
      n += old < r.l;
      nl = max(old, r.l);
    }
    if (r.u < seen.u) {
      const int old = atomicMin(&s[v].y, r.u);
      n += old > r.u;
      nu = min(old, r.u);
    }
    if (n && is_bot(mk(nl, nu))) failed = 1;
    return n;
  }
};

// A thread-private store (one propagator applied to its own three intervals).
struct LocalStore {
  Itv v[3];
  __device__ __forceinline__ Itv load(int i) const { return v[i]; }
  __device__ __forceinline__ int embed(int i, Itv, Itv r, int &failed) {
    int n = 0;
    if (r.l > v[i].l) { v[i].l = r.l; ++n; }
    if (r.u < v[i].u) { v[i].u = r.u; ++n; }
    if (n && is_bot(v[i])) failed = 1;
    return n;
  }
};

}  // namespace pirgpu
