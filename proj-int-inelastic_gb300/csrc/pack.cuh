// Column constants of the antipodal packing, shared by the CUDA-core and the
// tensor-core column passes.
#pragma once

#include "fft_reg.cuh"

namespace pii {

// Antipodal packing (the _PK column modes).  For a pair p and its antipode
// q = -sigma_p the phase and gain tables are conjugates, E_q = conj E_p and
// g_q = conj g_p (src/collision/inelastic_collisions.py:86-105).  With
// X+ = (X(k) + conj X(-k)) / 2 (X~(k) = conj X(-k) conjugates the factor of
// every Nyquist component, storage index n/2, which is its own negative), the
// real fields IFFT3(f^ E+_p) and IFFT3(f^ E+_q) pack into one complex pass on
// f^ t with the REAL phase t = Re E+_p + Im E+_p, and that pass's output F
// gives both pairs' gain terms (up to their Hermitian part, all that the real
// inverse transform of the sum keeps) as 2 s F, s = Re g+_p - Im g+_p.  The
// parts E - E+ and g - g+ live on the Nyquist planes only; the Nyquist
// correction adds what they contribute.  Per column j = (k_b, k_c) the
// separable rows give, for k_a != n/2,
//   t = e_a.x (c.x + c.y) + e_a.y (c.x - c.y),   c = (e_bc + e~_bc) / 2,
//   s = g_a.x (d.x - d.y) - g_a.y (d.x + d.y),   d = (g_bc + g~_bc) / 2,
// and at k_a = n/2 the two-term forms (e_a e_bc + conj e_a e~_bc) / 2 and
// (g_a g_bc + conj g_a g~_bc) / 2.
template <typename V>
__device__ __forceinline__ V cconj_v(V v) {
  v.y = -v.y;
  return v;
}
// (c.x + c.y, c.x - c.y, value at k_a = n/2) of the real phase t for column (jb, jc)
template <typename T, typename V, int NV>
__device__ __forceinline__ void pack_t_consts(const V* ep, int jb, int jc, T& cp, T& cm, T& th) {
  constexpr int H = NV / 2;
  const V eb = ep[NV + jb], ec = ep[2 * NV + jc];
  const V ebc = cmul(eb, ec);
  const V ebct = cmul(jb == H ? cconj_v(eb) : eb, jc == H ? cconj_v(ec) : ec);
  const T cx = T(0.5) * (ebc.x + ebct.x), cy = T(0.5) * (ebc.y + ebct.y);
  cp = cx + cy;
  cm = cx - cy;
  const V eh = ep[H];
  const V u = cmul(eh, ebc), w = cmul(cconj_v(eh), ebct);
  th = T(0.5) * (u.x + w.x + u.y + w.y);
}
// (d.x - d.y, d.x + d.y, value at k_a = n/2) of the real coefficient s for column (jb, jc)
template <typename T, typename V, int NV>
__device__ __forceinline__ void pack_s_consts(const V* gp, int jb, int jc, T& dp, T& dm, T& sh) {
  constexpr int H = NV / 2;
  const V gb = gp[NV + jb], gc = gp[2 * NV + jc];
  const V gbc = cmul(gb, gc);
  const V gbct = cmul(jb == H ? cconj_v(gb) : gb, jc == H ? cconj_v(gc) : gc);
  const T dx = T(0.5) * (gbc.x + gbct.x), dy = T(0.5) * (gbc.y + gbct.y);
  dp = dx - dy;
  dm = dx + dy;
  const V gh = gp[H];
  const V u = cmul(gh, gbc), w = cmul(cconj_v(gh), gbct);
  sh = T(0.5) * ((u.x + w.x) - (u.y + w.y));
}

}  // namespace pii
