// fmtfixed.cuh -- printf's "%.<prec>f" and "%d" for doubles and ints, on the
// device or the host (same source), byte for byte as glibc prints them.
//
// glibc formats the exact binary value of a double and rounds it to `prec`
// decimals half to even (the current rounding mode).  Here the value
// m * 2^e (m the 53-bit significand) is split into its integer part and its
// fraction; the fraction scaled by 10^prec is formed exactly in 128 bits
// (m < 2^53, 10^prec <= 10^17 < 2^57) and rounded half to even on the
// remainder, with the carry into the integer part.  Values of magnitude
// 2^63 and above are not handled (fmt_fixed returns -1); NaN and infinity
// print as "nan", "-nan", "inf", "-inf".  `width` pads on the left with
// spaces like printf's field width.
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define FMT_HD __host__ __device__ __forceinline__
#else
#define FMT_HD inline
#endif

namespace imdfmt {

typedef unsigned __int128 u128;

FMT_HD uint64_t double_bits(double v) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(v);
#else
  uint64_t b;
  memcpy(&b, &v, sizeof b);
  return b;
#endif
}

FMT_HD uint64_t pow10u(int p) {
  uint64_t r = 1;
  for (int k = 0; k < p; k++) r *= 10u;
  return r;
}

// decimal digits of v (at least `mind` of them, zero-padded) into out;
// returns the count
FMT_HD int put_uint(uint64_t v, int mind, char *out) {
  char tmp[24];
  int n = 0;
  do {
    tmp[n++] = (char)('0' + (int)(v % 10u));
    v /= 10u;
  } while (v);
  while (n < mind) tmp[n++] = '0';
  for (int k = 0; k < n; k++) out[k] = tmp[n - 1 - k];
  return n;
}

FMT_HD int pad_left(char *out, int len, int width) {
  if (len >= width) return len;
  const int sh = width - len;
  for (int k = len - 1; k >= 0; k--) out[k + sh] = out[k];
  for (int k = 0; k < sh; k++) out[k] = ' ';
  return width;
}

// printf("%*.*f", width, prec, v) into out (at most 22 + prec + width
// bytes, no terminating zero); returns the length, or -1 for |v| >= 2^63
FMT_HD int fmt_fixed(double v, int prec, int width, char *out) {
  const uint64_t bits = double_bits(v);
  const bool neg = (bits >> 63) != 0;
  const int ex = (int)((bits >> 52) & 0x7ffu);
  const uint64_t frac_bits = bits & ((1ull << 52) - 1u);
  int n = 0;
  if (ex == 0x7ff) {
    if (neg) out[n++] = '-';
    const char *w = frac_bits ? "nan" : "inf";
    for (int k = 0; k < 3; k++) out[n++] = w[k];
    return pad_left(out, n, width);
  }
  const uint64_t m = ex ? (frac_bits | (1ull << 52)) : frac_bits;
  const int e = ex ? ex - 1075 : -1074;  // v = m * 2^e
  uint64_t ip = 0;                        // integer part
  uint64_t fs = 0;                        // fraction * 10^prec, rounded
  const uint64_t scale = pow10u(prec);
  if (e >= 0) {
    if (e > 10) return -1;                // m * 2^e >= 2^63
    ip = m << e;
  } else {
    const int sh = -e;
    uint64_t f;                           // fraction = f * 2^-sh
    if (sh < 64) {
      ip = m >> sh;
      f = m & ((1ull << sh) - 1u);
    } else {
      ip = 0;
      f = m;
    }
    if (sh < 128) {
      const u128 p = (u128)f * scale;     // < 2^53 * 2^57
      u128 q = p >> sh;
      const u128 rem = p - (q << sh);
      const u128 half = (u128)1 << (sh - 1);
      // half to even on the last printed digit: the fraction's, or with no
      // decimals the integer part's
      const bool odd = prec ? (q & 1u) != 0 : (ip & 1u) != 0;
      if (rem > half || (rem == half && odd)) q += 1;
      fs = (uint64_t)q;
    } else {
      fs = 0;                             // below 2^-75: far under half a unit
    }
    if (fs >= scale) {                    // the rounding carried
      fs -= scale;
      ip += 1;
    }
  }
  if (neg) out[n++] = '-';
  n += put_uint(ip, 1, out + n);
  if (prec > 0) {
    out[n++] = '.';
    n += put_uint(fs, prec, out + n);
  }
  return pad_left(out, n, width);
}

// printf("%d", v)
FMT_HD int fmt_int(int v, char *out) {
  int n = 0;
  uint64_t u;
  if (v < 0) {
    out[n++] = '-';
    u = (uint64_t)(-(int64_t)v);
  } else {
    u = (uint64_t)v;
  }
  return n + put_uint(u, 1, out + n);
}

}  // namespace imdfmt
