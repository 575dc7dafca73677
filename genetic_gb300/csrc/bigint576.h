// 576-bit modular arithmetic for RANLUX jump-ahead (host and device).
//
// genetIC's white noise comes from RANLUX (GSL ranlxs2, called at
// genetIC/src/simulation/field/randomfieldgenerator.hpp:43-45,228-229).  RANLUX's
// subtract-with-borrow recurrence y_n = y_{n-10} - y_{n-24} - c_{n-1} (mod 2^24)
// is equivalent to a multiplicative congruential generator modulo
// m = 2^576 - 2^240 + 1 with multiplier a = 2^-24 mod m (Marsaglia & Zaman 1991;
// Tezuka, L'Ecuyer & Couture 1993).  The state (y_{n-24..n-1}, c) maps to
//   Y_n = (S - Z - c) mod m,  Z = sum_k 2^(24k) y_{n-24+k},  S = Z >> 336,
// and Y_{n+1} = a Y_n.  Jumping j steps ahead is one multiplication by a^j; the
// state is read back from V = -Y mod m = S (2^336 - 1) + T (T = low 336 bits of
// Z, borrow folded into T).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define GIC_HD __host__ __device__ __forceinline__
#else
#define GIC_HD inline
#endif

struct U576 {
  uint32_t w[18];  // little-endian 32-bit limbs
};

GIC_HD void u576_zero(U576 &a) {
  for (int i = 0; i < 18; ++i) a.w[i] = 0;
}

// m = 2^576 - 2^240 + 1: limbs 0 = 1, 1..6 = 0, 7 = 0xFFFF0000, 8..17 = 0xFFFFFFFF
GIC_HD uint32_t u576_mod_limb(int i) {
  return i == 0 ? 1u : (i < 7 ? 0u : (i == 7 ? 0xFFFF0000u : 0xFFFFFFFFu));
}

// r >= m ?
GIC_HD bool u576_ge_mod(const uint32_t *r, uint32_t top) {
  if (top) return true;
  for (int i = 17; i >= 0; --i) {
    uint32_t mi = u576_mod_limb(i);
    if (r[i] != mi) return r[i] > mi;
  }
  return true;
}

// r -= m, returns the borrow-adjusted top word
GIC_HD uint32_t u576_sub_mod(uint32_t *r, uint32_t top) {
  int64_t br = 0;
  for (int i = 0; i < 18; ++i) {
    int64_t v = (int64_t)r[i] - (int64_t)u576_mod_limb(i) + br;
    r[i] = (uint32_t)v;
    br = v >> 32;
  }
  return (uint32_t)((int64_t)top + br);
}

// Reduce x (nlimbs limbs, value < 2^(32 nlimbs), nlimbs <= 36) modulo m using
// 2^576 = 2^240 - 1 (mod m).  Result in r.
GIC_HD void u576_reduce(U576 &r, const uint32_t *x, int nlimbs) {
  uint32_t cur[36];
  int n = nlimbs;
  for (int i = 0; i < 36; ++i) cur[i] = i < n ? x[i] : 0u;
  while (n > 18) {
    // cur = L + H*2^576 -> L + (H << 240) - H ; H has (n-18) limbs
    int nh = n - 18;
    int64_t acc[36];
    for (int i = 0; i < 36; ++i) acc[i] = 0;
    for (int i = 0; i < 18; ++i) acc[i] += cur[i];
    for (int i = 0; i < nh; ++i) {
      uint64_t h = cur[18 + i];
      // h << 240 = h << (7*32 + 16)
      acc[i + 7] += (int64_t)((h << 16) & 0xFFFFFFFFull);
      acc[i + 8] += (int64_t)(h >> 16);
      acc[i] -= (int64_t)h;
    }
    int64_t carry = 0;
    int top = 0;
    for (int i = 0; i < 36; ++i) {
      int64_t v = acc[i] + carry;
      cur[i] = (uint32_t)v;
      carry = v >> 32;
      if (cur[i]) top = i + 1;
    }
    n = top < 18 ? 18 : top;
  }
  uint32_t hi = 0;
  for (int i = 0; i < 18; ++i) r.w[i] = cur[i];
  while (u576_ge_mod(r.w, hi)) hi = u576_sub_mod(r.w, hi);
}

GIC_HD void u576_mulmod(U576 &r, const U576 &a, const U576 &b) {
  uint32_t p[36];
  for (int i = 0; i < 36; ++i) p[i] = 0;
  for (int i = 0; i < 18; ++i) {
    uint64_t carry = 0;
    uint64_t ai = a.w[i];
    for (int j = 0; j < 18; ++j) {
      uint64_t t = ai * (uint64_t)b.w[j] + (uint64_t)p[i + j] + carry;
      p[i + j] = (uint32_t)t;
      carry = t >> 32;
    }
    p[i + 18] = (uint32_t)carry;
  }
  u576_reduce(r, p, 36);
}

// a = 2^-24 mod m = m - (m - 1)/2^24 = 2^576 - 2^552 - 2^240 + 2^216 + 1
GIC_HD void u576_ranlux_multiplier(U576 &a) {
  // build as m - ((m-1) >> 24); (m-1)>>24 = 2^552 - 2^216
  uint32_t t[19];
  for (int i = 0; i < 19; ++i) t[i] = 0;
  // m limbs
  for (int i = 0; i < 18; ++i) t[i] = u576_mod_limb(i);
  // subtract 2^552 (bit 552 = limb 17 bit 8) and add 2^216 (limb 6 bit 24)
  int64_t acc[18];
  for (int i = 0; i < 18; ++i) acc[i] = t[i];
  acc[17] -= (int64_t)1 << 8;
  acc[6] += (int64_t)1 << 24;
  int64_t carry = 0;
  for (int i = 0; i < 18; ++i) {
    int64_t v = acc[i] + carry;
    a.w[i] = (uint32_t)v;
    carry = v >> 32;
  }
}

// r = a^e mod m for a 64-bit exponent
GIC_HD void u576_powmod(U576 &r, const U576 &a, uint64_t e) {
  U576 base = a, acc;
  u576_zero(acc);
  acc.w[0] = 1;
  while (e) {
    if (e & 1) u576_mulmod(acc, acc, base);
    e >>= 1;
    if (e) u576_mulmod(base, base, base);
  }
  r = acc;
}

// 24-bit RANLUX state (oldest first, y[0] = y_{n-24}) with borrow c -> Y.
GIC_HD void u576_from_state(U576 &Y, const uint32_t *y, uint32_t c) {
  // Z = sum_k 2^(24k) y_k ; pack 24-bit digits into 32-bit limbs
  U576 Z;
  u576_zero(Z);
  for (int k = 0; k < 24; ++k) {
    int bit = 24 * k;
    int limb = bit >> 5, off = bit & 31;
    uint64_t v = (uint64_t)(y[k] & 0xFFFFFFu) << off;
    Z.w[limb] |= (uint32_t)v;
    if (limb + 1 < 18) Z.w[limb + 1] |= (uint32_t)(v >> 32);
  }
  // S = Z >> 336 (336 = 10*32 + 16), 240 bits
  U576 S;
  u576_zero(S);
  for (int i = 0; i < 8; ++i) {
    uint64_t lo = Z.w[10 + i];
    uint64_t hi = (11 + i) < 18 ? Z.w[11 + i] : 0u;
    S.w[i] = (uint32_t)(((hi << 32) | lo) >> 16);
  }
  // Zr = Z mod m (Z < 2^576, so at most one subtraction)
  uint32_t top = 0;
  U576 Zr = Z;
  if (u576_ge_mod(Zr.w, top)) u576_sub_mod(Zr.w, top);
  // Y = S - Zr - c  (mod m)
  int64_t br = 0;
  for (int i = 0; i < 18; ++i) {
    int64_t v = (int64_t)S.w[i] - (int64_t)Zr.w[i] - (i == 0 ? (int64_t)c : 0) + br;
    Y.w[i] = (uint32_t)v;
    br = v >> 32;
  }
  if (br < 0) {  // add m
    int64_t cy = 0;
    for (int i = 0; i < 18; ++i) {
      int64_t v = (int64_t)Y.w[i] + (int64_t)u576_mod_limb(i) + cy;
      Y.w[i] = (uint32_t)v;
      cy = v >> 32;
    }
  }
}

// Y -> equivalent 24-bit state (oldest first) with zero borrow.
GIC_HD void u576_to_state(uint32_t *y, const U576 &Y) {
  // V = (m - Y) mod m
  U576 V;
  bool yzero = true;
  for (int i = 0; i < 18; ++i) yzero = yzero && Y.w[i] == 0;
  if (yzero) {
    u576_zero(V);
  } else {
    int64_t br = 0;
    for (int i = 0; i < 18; ++i) {
      int64_t v = (int64_t)u576_mod_limb(i) - (int64_t)Y.w[i] + br;
      V.w[i] = (uint32_t)v;
      br = v >> 32;
    }
  }
  // V = Vhi * 2^336 + Vlo ; W = Vhi + Vlo ; S = Vhi (+1 per reduction of W)
  uint32_t vlo[12], vhi[8];
  for (int i = 0; i < 10; ++i) vlo[i] = V.w[i];
  vlo[10] = V.w[10] & 0xFFFFu;
  vlo[11] = 0;
  for (int i = 0; i < 8; ++i) {
    uint64_t lo = V.w[10 + i];
    uint64_t hi = (11 + i) < 18 ? V.w[11 + i] : 0u;
    vhi[i] = (uint32_t)(((hi << 32) | lo) >> 16);
  }
  uint32_t W[12];
  uint64_t cy = 0;
  for (int i = 0; i < 12; ++i) {
    uint64_t v = (uint64_t)vlo[i] + (i < 8 ? vhi[i] : 0u) + cy;
    W[i] = (uint32_t)v;
    cy = v >> 32;
  }
  uint32_t S[8];
  for (int i = 0; i < 8; ++i) S[i] = vhi[i];
  // while W >= 2^336 - 1 : W -= 2^336 - 1 ; S += 1
  for (int it = 0; it < 4; ++it) {
    // W >= 2^336 - 1  <=>  W + 1 >= 2^336  <=>  bits >= 336 set, or W == 2^336-1
    bool ge = (W[10] >> 16) != 0 || W[11] != 0;
    if (!ge) {
      bool allones = (W[10] & 0xFFFFu) == 0xFFFFu;
      for (int i = 0; i < 10 && allones; ++i) allones = W[i] == 0xFFFFFFFFu;
      ge = allones;
    }
    if (!ge) break;
    // W = W - 2^336 + 1
    int64_t acc = 1;
    for (int i = 0; i < 12; ++i) {
      int64_t v = (int64_t)W[i] + acc - (i == 10 ? (int64_t)0x10000 : 0);
      W[i] = (uint32_t)v;
      acc = v >> 32;
    }
    uint64_t c2 = 1;
    for (int i = 0; i < 8 && c2; ++i) {
      uint64_t v = (uint64_t)S[i] + c2;
      S[i] = (uint32_t)v;
      c2 = v >> 32;
    }
  }
  // Z' = S * 2^336 + W ; digits y_k = bits [24k, 24k+24)
  uint32_t Zp[18];
  for (int i = 0; i < 18; ++i) Zp[i] = 0;
  for (int i = 0; i < 11; ++i) Zp[i] = W[i];
  Zp[10] &= 0xFFFFu;
  for (int i = 0; i < 8; ++i) {
    uint64_t v = (uint64_t)S[i] << 16;
    Zp[10 + i] |= (uint32_t)v;
    if (11 + i < 18) Zp[11 + i] |= (uint32_t)(v >> 32);
  }
  for (int k = 0; k < 24; ++k) {
    int bit = 24 * k;
    int limb = bit >> 5, off = bit & 31;
    uint64_t v = (uint64_t)Zp[limb] >> off;
    if (limb + 1 < 18) v |= (uint64_t)Zp[limb + 1] << (32 - off);
    y[k] = (uint32_t)(v & 0xFFFFFFu);
  }
}

// Luescher's seeding: 31-bit shift register, 48 bits per 48-bit word, most
// significant first; word k splits into y[2k] (low 24) and y[2k+1] (high 24).
GIC_HD void ranlux_seed_state(uint32_t *y, unsigned long long seed) {
  int bits[31];
  long long s = (long long)(seed == 0 ? 1 : seed);
  int v = (int)(s & 0xFFFFFFFFLL);
  for (int k = 0; k < 31; ++k) {
    bits[k] = v % 2;
    v /= 2;
  }
  int ib = 0, jb = 18;
  for (int k = 0; k < 12; ++k) {
    uint64_t w = 0;
    for (int m = 0; m < 48; ++m) {
      w = 2 * w + (uint64_t)bits[ib];
      bits[ib] = (bits[ib] + bits[jb]) % 2;
      ib = (ib + 1) % 31;
      jb = (jb + 1) % 31;
    }
    y[2 * k] = (uint32_t)(w & 0xFFFFFFu);
    y[2 * k + 1] = (uint32_t)(w >> 24);
  }
}
