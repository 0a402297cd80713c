// Matrix pools of one parameter point, built natively (host code).
//
// A plan's fused ops are products of the circuit's gate matrices; the
// planner records, per op, a recipe of steps (take a gate, widen by identity
// or selector bits, multiply a gate in, scale rows by a diagonal, ...).  For
// a new parameter point the pool is those recipes replayed on the point's
// gate matrices.  The planner's numpy replay runs every step as a few numpy
// calls; for one point of a plan with ~1000 ops that is ~10 ms of
// interpreter overhead, paid on every call of a parameterised circuit (every
// adjoint gradient).  Here the same steps run as plain loops over complex128
// values, then the pool is rounded to complex64 (the caller zeroes residues
// below 1e-12 as for the numpy pools).
//
// Program (int32 words), per pool entry:
//   kind (0 dense, 1 diag, 2 probe, 3 probe diag), offset (2 words, lo/hi),
//   then
//   dense:      ns, d, has_perm, [perm: d words], nsteps, steps...
//   diag:       nsteps, steps...
//   probe:      gate, d, has_perm, [perm: d words]
//   probe diag: gate
// Steps: 1 init_dense(gate) | 2 tx(n) | 3 sx(n) | 4 s2t(i) |
//        5 mul(gate, npos, pos...) | 6 dmul(gate, nb, tpos[nb], spos[nb]) |
//        7 diag_as_dense(nsub, sub steps..., nb, bits[nb], ntg, tg[ntg],
//                        nsl, sl[nsl]) |
//        8 init_diag(gate) | 9 dx(n) | 10 dd(gate, npos, pos...)
// (-1 in tpos / spos marks "not a target" / "not a selector").

#include <stdint.h>
#include <string.h>

#include <complex>
#include <string>
#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "gbq_internal.cuh"

namespace gbq {
namespace {

using cd = std::complex<double>;

// (a.re b.re - a.im b.im, a.re b.im + a.im b.re): the value std::complex's
// operator* returns for finite operands, without its library call for the
// infinite / NaN cases (every pool entry is finite)
static inline cd cmul(const cd& a, const cd& b) {
  return cd(a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real());
}

struct Gates {
  const cd* base;
  const int64_t* off;
  const int32_t* dim;
  int n;
  const cd* at(int gi) const { return base + off[gi]; }
};

struct Reader {
  const int32_t* p;
  const int32_t* end;
  bool ok = true;
  int next() {
    if (p >= end) {
      ok = false;
      return 0;
    }
    return *p++;
  }
};

struct Dense {
  int ns = 1, d = 1;
  std::vector<cd> m{cd(1.0, 0.0)};  // [ns][d][d]
};

static bool gate_ok(const Gates& g, int gi) { return gi >= 0 && gi < g.n; }

static void run_diag_steps(Reader& r, int nsteps, const Gates& g, std::vector<cd>& D) {
  D.assign(1, cd(1.0, 0.0));
  for (int s = 0; s < nsteps && r.ok; ++s) {
    const int kind = r.next();
    if (kind == 8) {  // init_diag
      const int gi = r.next();
      if (!gate_ok(g, gi)) return void(r.ok = false);
      const int dg = g.dim[gi];
      const cd* G = g.at(gi);
      D.resize(dg);
      for (int i = 0; i < dg; ++i) D[i] = G[(int64_t)i * dg + i];
    } else if (kind == 9) {  // dx: new highest bits
      const int n = r.next();
      if (n < 0 || n > 20) return void(r.ok = false);
      const size_t len = D.size();
      std::vector<cd> out(len << n);
      for (size_t c = 0; c < ((size_t)1 << n); ++c)
        for (size_t x = 0; x < len; ++x) out[c * len + x] = D[x];
      D.swap(out);
    } else if (kind == 10) {  // dd: multiply by a diagonal gate on bit positions
      const int gi = r.next(), np = r.next();
      if (!gate_ok(g, gi) || np < 0 || np > 20) return void(r.ok = false);
      std::vector<int> pos(np);
      for (int i = 0; i < np; ++i) pos[i] = r.next();
      const int dg = g.dim[gi];
      const cd* G = g.at(gi);
      for (size_t x = 0; x < D.size(); ++x) {
        int sub = 0;
        for (int i = 0; i < np; ++i) sub |= (int)((x >> pos[i]) & 1) << i;
        if (sub >= dg) return void(r.ok = false);
        D[x] = cmul(D[x], G[(int64_t)sub * dg + sub]);
      }
    } else {
      r.ok = false;
    }
  }
}

static void run_dense_steps(Reader& r, int nsteps, const Gates& g, Dense& M) {
  for (int s = 0; s < nsteps && r.ok; ++s) {
    const int kind = r.next();
    switch (kind) {
      case 1: {  // init_dense
        const int gi = r.next();
        if (!gate_ok(g, gi)) return void(r.ok = false);
        const int d = g.dim[gi];
        M.ns = 1;
        M.d = d;
        M.m.assign(g.at(gi), g.at(gi) + (int64_t)d * d);
        break;
      }
      case 2: {  // tx: n identity target bits above the current ones
        const int n = r.next();
        if (n < 0 || n > 10) return void(r.ok = false);
        const int d = M.d, e = 1 << n, nd = d * e;
        std::vector<cd> out((size_t)M.ns * nd * nd);
        for (int sx = 0; sx < M.ns; ++sx)
          for (int a = 0; a < e; ++a)
            for (int i = 0; i < d; ++i)
              for (int j = 0; j < d; ++j)
                out[((size_t)sx * nd + a * d + i) * nd + a * d + j] = M.m[((size_t)sx * d + i) * d + j];
        M.d = nd;
        M.m.swap(out);
        break;
      }
      case 3: {  // sx: n selector bits above the current ones (copies)
        const int n = r.next();
        if (n < 0 || n > 10) return void(r.ok = false);
        const size_t blk = (size_t)M.ns * M.d * M.d;
        std::vector<cd> out(blk << n);
        for (size_t c = 0; c < ((size_t)1 << n); ++c) memcpy(&out[c * blk], M.m.data(), blk * sizeof(cd));
        M.ns <<= n;
        M.m.swap(out);
        break;
      }
      case 4: {  // s2t: selector i becomes the new highest target bit
        const int i = r.next();
        if (i < 0 || (1 << i) >= M.ns) return void(r.ok = false);
        const int ns2 = M.ns / 2, d = M.d, nd = 2 * d;
        std::vector<cd> out((size_t)ns2 * nd * nd, cd(0.0, 0.0));
        for (int q = 0; q < ns2; ++q) {
          const int keep = (q & ((1 << i) - 1)) | ((q >> i) << (i + 1));
          const int hi = keep | (1 << i);
          for (int a = 0; a < d; ++a)
            for (int b = 0; b < d; ++b) {
              out[((size_t)q * nd + a) * nd + b] = M.m[((size_t)keep * d + a) * d + b];
              out[((size_t)q * nd + d + a) * nd + d + b] = M.m[((size_t)hi * d + a) * d + b];
            }
        }
        M.ns = ns2;
        M.d = nd;
        M.m.swap(out);
        break;
      }
      case 5: {  // mul: left-multiply a gate acting on target positions
        const int gi = r.next(), np = r.next();
        if (!gate_ok(g, gi) || np < 1 || np > 10) return void(r.ok = false);
        std::vector<int> pos(np);
        int mask = 0;
        for (int k = 0; k < np; ++k) {
          pos[k] = r.next();
          if (pos[k] < 0 || (1 << pos[k]) >= M.d) return void(r.ok = false);
          mask |= 1 << pos[k];
        }
        const int d = M.d, dg = g.dim[gi];
        const cd* G = g.at(gi);
        std::vector<int> sub(d);
        for (int x = 0; x < d; ++x) {
          int v = 0;
          for (int k = 0; k < np; ++k) v |= ((x >> pos[k]) & 1) << k;
          if (v >= dg) return void(r.ok = false);
          sub[x] = v;
        }
        // F[r][c] = G[sub r][sub c] where r and c agree outside pos
        std::vector<cd> F((size_t)d * d, cd(0.0, 0.0));
        for (int a = 0; a < d; ++a)
          for (int b = 0; b < d; ++b)
            if ((a & ~mask) == (b & ~mask)) F[(size_t)a * d + b] = G[(int64_t)sub[a] * dg + sub[b]];
        std::vector<cd> out((size_t)M.ns * d * d);
        for (int sx = 0; sx < M.ns; ++sx) {
          const cd* m = &M.m[(size_t)sx * d * d];
          cd* o = &out[(size_t)sx * d * d];
          // F[a][b] is zero unless a and b agree outside the gate's bits:
          // sum only those b (ascending, as a dense product would), which
          // leaves out exact-zero terms alone
          for (int a = 0; a < d; ++a) {
            const int base = a & ~mask;
            for (int c = 0; c < d; ++c) {
              cd acc(0.0, 0.0);
              for (int t = 0;; t = (t - mask) & mask) {
                const int b = base | t;
                acc += cmul(F[(size_t)a * d + b], m[(size_t)b * d + c]);
                if (t == mask) break;
              }
              o[(size_t)a * d + c] = acc;
            }
          }
        }
        M.m.swap(out);
        break;
      }
      case 6: {  // dmul: scale rows by a diagonal gate over (targets, selectors)
        const int gi = r.next(), nb = r.next();
        if (!gate_ok(g, gi) || nb < 1 || nb > 10) return void(r.ok = false);
        std::vector<int> tpos(nb), spos(nb);
        for (int j = 0; j < nb; ++j) tpos[j] = r.next();
        for (int j = 0; j < nb; ++j) spos[j] = r.next();
        const int d = M.d, dg = g.dim[gi];
        const cd* G = g.at(gi);
        for (int sx = 0; sx < M.ns; ++sx)
          for (int a = 0; a < d; ++a) {
            int v = 0;
            for (int j = 0; j < nb; ++j) {
              const int bit = tpos[j] >= 0 ? (a >> tpos[j]) & 1 : (sx >> spos[j]) & 1;
              v |= bit << j;
            }
            if (v >= dg) return void(r.ok = false);
            const cd f = G[(int64_t)v * dg + v];
            cd* row = &M.m[((size_t)sx * d + a) * d];
            for (int c = 0; c < d; ++c) row[c] = cmul(row[c], f);
          }
        break;
      }
      case 7: {  // diag_as_dense
        const int nsub = r.next();
        std::vector<cd> D;
        run_diag_steps(r, nsub, g, D);
        const int nb = r.next();
        if (!r.ok || nb < 0 || nb > 16) return void(r.ok = false);
        std::vector<int> bits(nb);
        for (int j = 0; j < nb; ++j) bits[j] = r.next();
        const int ntg = r.next();
        if (ntg < 0 || ntg > 10) return void(r.ok = false);
        std::vector<int> tg(ntg);
        for (int j = 0; j < ntg; ++j) tg[j] = r.next();
        const int nsl = r.next();
        if (nsl < 0 || nsl > 10) return void(r.ok = false);
        std::vector<int> sl(nsl);
        for (int j = 0; j < nsl; ++j) sl[j] = r.next();
        const int ns = 1 << nsl, dt = 1 << ntg;
        Dense out;
        out.ns = ns;
        out.d = dt;
        out.m.assign((size_t)ns * dt * dt, cd(0.0, 0.0));
        for (int sx = 0; sx < ns; ++sx)
          for (int t = 0; t < dt; ++t) {
            int v = 0;
            for (int j = 0; j < nb; ++j) {
              int bit = 0, found = 0;
              for (int k = 0; k < ntg; ++k)
                if (tg[k] == bits[j]) bit = (t >> k) & 1, found = 1;
              if (!found)
                for (int k = 0; k < nsl; ++k)
                  if (sl[k] == bits[j]) bit = (sx >> k) & 1, found = 1;
              v |= bit << j;
            }
            if ((size_t)v >= D.size()) return void(r.ok = false);
            out.m[((size_t)sx * dt + t) * dt + t] = D[v];
          }
        M = std::move(out);
        break;
      }
      default:
        return void(r.ok = false);
    }
  }
}

// Pool entries as complex64, with real and imaginary parts whose magnitude
// is below 1e-12 (compared on the float32 bit pattern) stored as +0: the
// planner's snap of the numpy replay, so that both give the same bits.
static float snapped(double x) {
  static const uint32_t kSnap = [] {
    const float f = 1e-12f;
    uint32_t b;
    memcpy(&b, &f, 4);
    return b;
  }();
  const float f = (float)x;
  uint32_t b;
  memcpy(&b, &f, 4);
  return (b & 0x7fffffffu) < kSnap ? 0.0f : f;
}

static void put(gbq_c64* out, int64_t len, int64_t off, const std::vector<cd>& v, bool& ok) {
  if (off < 0 || off + (int64_t)v.size() > len) {
    ok = false;
    return;
  }
  for (size_t i = 0; i < v.size(); ++i) {
    out[off + i].re = snapped(v[i].real());
    out[off + i].im = snapped(v[i].imag());
  }
}

}  // namespace
}  // namespace gbq

using namespace gbq;

extern "C" int gbq_pool_build(const int32_t* prog, int64_t prog_len, const double* gates, const int64_t* gate_off,
                              const int32_t* gate_dim, int ngates, gbq_c64* out, int64_t pool_len) {
  if (!prog || prog_len < 0 || (ngates && (!gates || !gate_off || !gate_dim)) || !out || pool_len < 0)
    return GBQ_ERR_ARG;
  Gates g{reinterpret_cast<const cd*>(gates), gate_off, gate_dim, ngates};
  memset(out, 0, (size_t)pool_len * sizeof(gbq_c64));
  Reader r{prog, prog + prog_len};
  bool ok = true;
  while (r.ok && ok && r.p < r.end) {
    const int kind = r.next();
    const int64_t off = (int64_t)(uint32_t)r.next() | ((int64_t)r.next() << 32);
    if (kind == 0) {
      const int ns = r.next(), d = r.next(), has_perm = r.next();
      std::vector<int> perm;
      if (has_perm) {
        if (d < 1 || d > 64) return GBQ_ERR_ARG;
        perm.resize(d);
        for (int i = 0; i < d; ++i) perm[i] = r.next();
      }
      const int nsteps = r.next();
      Dense M;
      run_dense_steps(r, nsteps, g, M);
      if (!r.ok || M.ns != ns || M.d != d) return GBQ_ERR_ARG;
      if (has_perm) {
        std::vector<cd> pm(M.m.size());
        for (int sx = 0; sx < ns; ++sx)
          for (int a = 0; a < d; ++a)
            for (int b = 0; b < d; ++b) {
              if (perm[a] < 0 || perm[a] >= d || perm[b] < 0 || perm[b] >= d) return GBQ_ERR_ARG;
              pm[((size_t)sx * d + a) * d + b] = M.m[((size_t)sx * d + perm[a]) * d + perm[b]];
            }
        M.m.swap(pm);
      }
      put(out, pool_len, off, M.m, ok);
    } else if (kind == 1) {
      const int nsteps = r.next();
      std::vector<cd> D;
      run_diag_steps(r, nsteps, g, D);
      if (!r.ok) return GBQ_ERR_ARG;
      put(out, pool_len, off, D, ok);
    } else if (kind == 2 || kind == 3) {
      const int gi = r.next();
      if (gi < 0 || gi >= ngates) return GBQ_ERR_ARG;
      const int dg = gate_dim[gi];
      const cd* G = g.at(gi);
      std::vector<cd> v;
      if (kind == 3) {
        v.resize(dg);
        for (int i = 0; i < dg; ++i) v[i] = G[(int64_t)i * dg + i];
      } else {
        const int d = r.next(), has_perm = r.next();
        if (d != dg) return GBQ_ERR_ARG;
        std::vector<int> perm(d);
        for (int i = 0; i < d; ++i) perm[i] = has_perm ? r.next() : i;
        v.resize((size_t)d * d);
        for (int a = 0; a < d; ++a)
          for (int b = 0; b < d; ++b) {
            if (perm[a] < 0 || perm[a] >= d || perm[b] < 0 || perm[b] >= d) return GBQ_ERR_ARG;
            v[(size_t)a * d + b] = G[(int64_t)perm[a] * d + perm[b]];
          }
      }
      put(out, pool_len, off, v, ok);
    } else {
      return GBQ_ERR_ARG;
    }
  }
  return (r.ok && ok) ? GBQ_OK : GBQ_ERR_ARG;
}

extern "C" int gbq_pool_build_points(const int32_t* prog, int64_t prog_len, const double* gates, int64_t gate_stride,
                                     const int64_t* gate_off, const int32_t* gate_dim, int ngates, int npoints,
                                     gbq_c64* out, int64_t pool_len, int nthreads) {
  if (npoints < 0 || gate_stride < 0 || (npoints && !out) || (npoints && ngates && !gates)) return GBQ_ERR_ARG;
  if (npoints == 0) return GBQ_OK;
  int nt = nthreads > 0 ? nthreads : (int)std::thread::hardware_concurrency();
  nt = std::max(1, std::min({nt, npoints, 64}));
  std::atomic<int> next{0};
  std::atomic<int> rc{GBQ_OK};
  auto work = [&]() {
    for (;;) {
      const int p = next.fetch_add(1);
      if (p >= npoints || rc.load() != GBQ_OK) break;
      const int r = gbq_pool_build(prog, prog_len, gates + 2 * gate_stride * (int64_t)p, gate_off, gate_dim, ngates,
                                   out + pool_len * (int64_t)p, pool_len);
      if (r != GBQ_OK) rc.store(r);
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(work);
  work();
  for (auto& th : pool) th.join();
  return rc.load();
}

