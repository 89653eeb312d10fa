// Host-side scene numerics: GLL nodes, FP64 modal fits, the seeded synthetic
// scene generator, record packing and the Modified-A -> Bernstein change of
// basis used for rigorous hull boxes.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <thread>

#include "ho_host.h"

namespace ho {

// ---- PCG64 (XSL-RR 128/64, the published "pcg64" member of the PCG family)
static const unsigned __int128 kPcgMult =
    (static_cast<unsigned __int128>(0x2360ED051FC65DA4ULL) << 64) | 0x4385DF649FCCF645ULL;

Pcg64::Pcg64(uint64_t seed, uint64_t stream) {
  state = 0;
  inc = (static_cast<unsigned __int128>(stream) << 1) | 1u;
  next();
  state += seed;
  next();
}

uint64_t Pcg64::next() {
  const unsigned __int128 old = state;
  state = old * kPcgMult + inc;
  const uint64_t x = static_cast<uint64_t>(old >> 64) ^ static_cast<uint64_t>(old);
  const unsigned rot = static_cast<unsigned>(old >> 122);
  return (x >> rot) | (x << ((64u - rot) & 63u));
}

double Pcg64::uniform() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }

// ---- 1-D basis in FP64 -----------------------------------------------------
// Jacobi P^{(1,1)}_m by its three-term recurrence and the Modified-A modes
// built from it (the alpha = beta = 1 case of FEM-AABB/fem/ModalBasis.cuh).
static void jac11(int m, double x, double& p, double& dp) {
  double pm2 = 1.0, pm1 = 2.0 * x, qm2 = 0.0, qm1 = 2.0;
  if (m == 0) {
    p = 1.0;
    dp = 0.0;
    return;
  }
  if (m == 1) {
    p = pm1;
    dp = qm1;
    return;
  }
  for (int k = 2; k <= m; ++k) {
    const double A = double((2 * k + 1) * (k + 1)) / double(k * (k + 2));
    const double B = double(k + 1) / double(k + 2);
    const double pk = A * x * pm1 - B * pm2;
    const double qk = A * (pm1 + x * qm1) - B * qm2;
    pm2 = pm1;
    pm1 = pk;
    qm2 = qm1;
    qm1 = qk;
  }
  p = pm1;
  dp = qm1;
}

double mod_a(int i, double x) {
  if (i == 0) return 0.5 * (1.0 - x);
  if (i == 1) return 0.5 * (1.0 + x);
  double p, dp;
  jac11(i - 2, x, p, dp);
  return 0.25 * (1.0 - x * x) * p;
}

double mod_a_prime(int i, double x) {
  if (i == 0) return -0.5;
  if (i == 1) return 0.5;
  double p, dp;
  jac11(i - 2, x, p, dp);
  return -0.5 * x * p + 0.25 * (1.0 - x * x) * dp;
}

// Legendre P_N and P_N' by recurrence.
static void legendre(int N, double x, double& p, double& dp) {
  double p0 = 1.0, p1 = x;
  if (N == 0) {
    p = 1.0;
    dp = 0.0;
    return;
  }
  for (int k = 2; k <= N; ++k) {
    const double pk = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    p0 = p1;
    p1 = pk;
  }
  p = p1;
  dp = N * (x * p1 - p0) / (x * x - 1.0);
}

// GLL nodes: -1, the roots of P'_{n-1}, +1. Newton on P'_{N} using
// P''_N = (2x P'_N - N(N+1) P_N)/(1-x^2), from Chebyshev-Lobatto guesses.
std::vector<double> gll_nodes(int n) {
  std::vector<double> x(n);
  if (n == 1) {
    x[0] = 0.0;
    return x;
  }
  const int N = n - 1;
  x[0] = -1.0;
  x[n - 1] = 1.0;
  for (int i = 1; i < N; ++i) {
    double t = -std::cos(M_PI * i / N);
    for (int it = 0; it < 100; ++it) {
      double p, dp;
      legendre(N, t, p, dp);
      const double d2p = (2.0 * t * dp - N * (N + 1.0) * p) / (1.0 - t * t);
      const double step = dp / d2p;
      t -= step;
      if (std::fabs(step) < 1e-16) break;
    }
    x[i] = t;
  }
  for (int i = 0; i < n / 2; ++i) {  // exact antisymmetry
    const double m = 0.5 * (x[n - 1 - i] - x[i]);
    x[i] = -m;
    x[n - 1 - i] = m;
  }
  if (n % 2) x[n / 2] = 0.0;
  return x;
}

static bool invert_dense(std::vector<double> a, int n, std::vector<double>& inv) {
  inv.assign(static_cast<size_t>(n) * n, 0.0);
  for (int i = 0; i < n; ++i) inv[i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(a[r * n + c]) > std::fabs(a[piv * n + c])) piv = r;
    if (std::fabs(a[piv * n + c]) < 1e-300) return false;
    if (piv != c)
      for (int k = 0; k < n; ++k) {
        std::swap(a[c * n + k], a[piv * n + k]);
        std::swap(inv[c * n + k], inv[piv * n + k]);
      }
    const double s = 1.0 / a[c * n + c];
    for (int k = 0; k < n; ++k) {
      a[c * n + k] *= s;
      inv[c * n + k] *= s;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = a[r * n + c];
      if (f == 0.0) continue;
      for (int k = 0; k < n; ++k) {
        a[r * n + k] -= f * a[c * n + k];
        inv[r * n + k] -= f * inv[c * n + k];
      }
    }
  }
  return true;
}

bool modal_vandermonde_inverse(const std::vector<double>& nodes, std::vector<double>& inv) {
  const int n = static_cast<int>(nodes.size());
  std::vector<double> V(static_cast<size_t>(n) * n);
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) V[r * n + c] = mod_a(c, nodes[r]);
  return invert_dense(V, n, inv);
}

// modal[c,b,a] = sum_{k,j,i} Vinv[a,i] Vinv[b,j] Vinv[c,k] nodal[k,j,i]
// (the same per-direction solve as FEM-AABB/xml_fld_math.cpp:379-483).
void tensor_modal_fit(int n, const std::vector<double>& vinv, const double* nodal, double* modal) {
  const size_t S = static_cast<size_t>(n) * n * n;
  std::vector<double> t1(S), t2(S);
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int a = 0; a < n; ++a) {
        double s = 0;
        for (int i = 0; i < n; ++i) s += vinv[a * n + i] * nodal[(k * n + j) * n + i];
        t1[(k * n + j) * n + a] = s;
      }
  for (int k = 0; k < n; ++k)
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a) {
        double s = 0;
        for (int j = 0; j < n; ++j) s += vinv[b * n + j] * t1[(k * n + j) * n + a];
        t2[(k * n + b) * n + a] = s;
      }
  for (int c = 0; c < n; ++c)
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a) {
        double s = 0;
        for (int k = 0; k < n; ++k) s += vinv[c * n + k] * t2[(k * n + b) * n + a];
        modal[(c * n + b) * n + a] = s;
      }
}

// ---- the host modal fitter ----------------------------------------------------
namespace {
class HostFitter final : public ModalFitter {
 public:
  bool add(const double* nodal, int comps, int nx, int ny, int nz, std::vector<float>* dst, int64_t dst_off) override {
    for (int n : {nx, ny, nz}) {
      if (n < 1 || n > kMaxModes) return false;
      if (vinv_[n].empty() && !modal_vandermonde_inverse(gll_nodes(n), vinv_[n])) return false;
    }
    const std::vector<double>&vr = vinv_[nx], &vs = vinv_[ny], &vt = vinv_[nz];
    const size_t S = static_cast<size_t>(nx) * ny * nz;
    auto idx = [&](int i, int j, int k) { return (static_cast<size_t>(k) * ny + j) * nx + i; };
    b_.resize(S);
    d_.resize(S);
    for (int c = 0; c < comps; ++c) {
      const double* a = nodal + c * S;
      for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
          for (int m = 0; m < nx; ++m) {
            double s = 0;
            for (int i = 0; i < nx; ++i) s += vr[m * nx + i] * a[idx(i, j, k)];
            b_[idx(m, j, k)] = s;
          }
      for (int k = 0; k < nz; ++k)
        for (int m = 0; m < ny; ++m)
          for (int i = 0; i < nx; ++i) {
            double s = 0;
            for (int j = 0; j < ny; ++j) s += vs[m * ny + j] * b_[idx(i, j, k)];
            d_[idx(i, m, k)] = s;
          }
      for (int m = 0; m < nz; ++m)
        for (int j = 0; j < ny; ++j)
          for (int i = 0; i < nx; ++i) {
            double s = 0;
            for (int k = 0; k < nz; ++k) s += vt[m * nz + k] * d_[idx(i, j, k)];
            (*dst)[dst_off + c * S + idx(i, j, m)] = static_cast<float>(s);
          }
    }
    return true;
  }
  bool finish() override { return true; }

 private:
  std::vector<double> vinv_[kMaxModes + 1];
  std::vector<double> b_, d_;
};
}  // namespace

std::unique_ptr<ModalFitter> make_host_fitter() { return std::make_unique<HostFitter>(); }

// ---- synthetic scenes -------------------------------------------------------
template <class F>
static void parallel_chunks(int64_t n, F&& fn) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int nt = static_cast<int>(std::min<int64_t>(hw, std::max<int64_t>(1, n / 64)));
  if (nt <= 1) {
    fn(0, n);
    return;
  }
  std::atomic<int64_t> next{0};
  std::vector<std::thread> pool;
  for (int t = 0; t < nt; ++t)
    pool.emplace_back([&] {
      for (;;) {
        const int64_t b = next.fetch_add(32);
        if (b >= n) break;
        fn(b, std::min(n, b + 32));
      }
    });
  for (auto& th : pool) th.join();
}

int generate_synthetic(const ho_synth_params& p, HostScene& hs, std::string& err) {
  if (p.nx <= 0 || p.ny <= 0 || p.nz <= 0) {
    err = "synthetic grid dimensions must be positive";
    return HO_ERR_ARG;
  }
  if (p.order_min < kMinModes - 1 || p.order_max > kMaxModes - 1 || p.order_min > p.order_max) {
    err = "synthetic order range must satisfy 1 <= order_min <= order_max <= 8";
    return HO_ERR_RANGE;
  }
  if (p.n_gauss < 0) {
    err = "n_gauss must be >= 0";
    return HO_ERR_ARG;
  }
  const int64_t ne = static_cast<int64_t>(p.nx) * p.ny * p.nz;
  // Gaussians first from stream 1, then per-element orders from stream 2.
  Pcg64 rg(p.seed, 1);
  std::vector<double> gc(3 * p.n_gauss), gs(p.n_gauss), ga(p.n_gauss);
  for (int g = 0; g < p.n_gauss; ++g) {
    gc[3 * g] = rg.uniform();
    gc[3 * g + 1] = rg.uniform();
    gc[3 * g + 2] = rg.uniform();
    gs[g] = 0.1 + 0.2 * rg.uniform();
    ga[g] = -1.0 + 2.0 * rg.uniform();
  }
  std::vector<int> order(ne, p.order_min);
  if (p.order_max > p.order_min) {
    Pcg64 ro(p.seed, 2);
    const int span = p.order_max - p.order_min + 1;
    for (int64_t e = 0; e < ne; ++e)
      order[e] = p.order_min + std::min(span - 1, static_cast<int>(ro.uniform() * span));
  }
  const double hx = 1.0 / p.nx, hy = 1.0 / p.ny, hz = 1.0 / p.nz;
  const double h = std::min(hx, std::min(hy, hz));
  const double amp = p.curve_amp * h;
  const double two_pi = 2.0 * M_PI;
  auto disp = [&](double x, double y, double z) {
    return amp * std::sin(two_pi * x) * std::sin(two_pi * y) * std::sin(two_pi * z);
  };

  // offsets (serial, so the layout does not depend on threading)
  const int64_t base = hs.size();
  int64_t gpos = static_cast<int64_t>(hs.geom.size()), fpos = static_cast<int64_t>(hs.field.size());
  hs.corners.resize((base + ne) * 24);
  hs.gmodes.resize((base + ne) * 3);
  hs.fmodes.resize((base + ne) * 3);
  hs.goff.resize(base + ne);
  hs.foff.resize(base + ne);
  for (int64_t e = 0; e < ne; ++e) {
    const int n = order[e] + 1;
    const int64_t S = static_cast<int64_t>(n) * n * n;
    hs.goff[base + e] = gpos;
    hs.foff[base + e] = fpos;
    gpos += 3 * S;
    fpos += S;
    for (int a = 0; a < 3; ++a) {
      hs.gmodes[(base + e) * 3 + a] = n;
      hs.fmodes[(base + e) * 3 + a] = n;
    }
  }
  hs.geom.resize(gpos);
  hs.field.resize(fpos);

  std::vector<std::vector<double>> nodes(kMaxModes + 1), vinv(kMaxModes + 1);
  for (int n = kMinModes; n <= kMaxModes; ++n) {
    nodes[n] = gll_nodes(n);
    if (!modal_vandermonde_inverse(nodes[n], vinv[n])) {
      err = "singular modal Vandermonde";
      return HO_ERR_ARG;
    }
  }

  parallel_chunks(ne, [&](int64_t b, int64_t eend) {
    std::vector<double> nodal(4 * kMaxModes * kMaxModes * kMaxModes), modal(kMaxModes * kMaxModes * kMaxModes);
    for (int64_t e = b; e < eend; ++e) {
      const int kx = static_cast<int>(e % p.nx), ky = static_cast<int>((e / p.nx) % p.ny),
                kz = static_cast<int>(e / (static_cast<int64_t>(p.nx) * p.ny));
      const int n = order[e] + 1;
      const int S = n * n * n;
      const std::vector<double>& r = nodes[n];
      double* nx_ = nodal.data();
      double* ny_ = nx_ + S;
      double* nz_ = ny_ + S;
      double* nf_ = nz_ + S;
      for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i) {
            const double X = (kx + 0.5 * (r[i] + 1.0)) * hx;
            const double Y = (ky + 0.5 * (r[j] + 1.0)) * hy;
            const double Z = (kz + 0.5 * (r[k] + 1.0)) * hz;
            const double dl = disp(X, Y, Z);
            const double x = X + dl, y = Y + dl, z = Z + dl;
            double u = 0.0;
            for (int g = 0; g < p.n_gauss; ++g) {
              const double dx = x - gc[3 * g], dy = y - gc[3 * g + 1], dz = z - gc[3 * g + 2];
              u += ga[g] * std::exp(-(dx * dx + dy * dy + dz * dz) / (2.0 * gs[g] * gs[g]));
            }
            const int q = (k * n + j) * n + i;
            nx_[q] = x;
            ny_[q] = y;
            nz_[q] = z;
            nf_[q] = u;
          }
      float* gdst = hs.geom.data() + hs.goff[base + e];
      for (int c = 0; c < 3; ++c) {
        tensor_modal_fit(n, vinv[n], nodal.data() + c * S, modal.data());
        for (int q = 0; q < S; ++q) gdst[c * S + q] = static_cast<float>(modal[q]);
      }
      tensor_modal_fit(n, vinv[n], nf_, modal.data());
      float* fdst = hs.field.data() + hs.foff[base + e];
      for (int q = 0; q < S; ++q) fdst[q] = static_cast<float>(modal[q]);
      // displaced corners, XML order: (0,0,0) (1,0,0) (1,1,0) (0,1,0) then z = 1
      static const int cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1},
                       cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
      float* cd = hs.corners.data() + (base + e) * 24;
      for (int v = 0; v < 8; ++v) {
        const double X = (kx + cx[v]) * hx, Y = (ky + cy[v]) * hy, Z = (kz + cz[v]) * hz;
        const double dl = disp(X, Y, Z);
        cd[3 * v] = static_cast<float>(X + dl);
        cd[3 * v + 1] = static_cast<float>(Y + dl);
        cd[3 * v + 2] = static_cast<float>(Z + dl);
      }
    }
  });
  return HO_OK;
}

int scene_max_modes(const HostScene& hs) {
  int m = 0;
  for (int64_t e = 0; e < hs.size(); ++e) {
    for (int a = 0; a < 3; ++a) {
      const int g = hs.goff[e] >= 0 ? static_cast<int>(hs.gmodes[3 * e + a]) : 2;
      m = std::max(m, g);
      if (hs.foff[e] >= 0) m = std::max(m, static_cast<int>(hs.fmodes[3 * e + a]));
    }
  }
  return std::max(m, 2);
}

// XML vertex v sits at Z-order corner (i + 2j + 4k) kXml2Z[v]
// (FEM-AABB/fem/HexElement.cu:107-109); the map is its own inverse.
static const int kXml2Z[8] = {0, 1, 3, 2, 4, 5, 7, 6};

// Cube order of element e: its largest geometry or field modes count per
// direction (a trilinear element counts as 2).
int element_order(const HostScene& hs, int64_t e) {
  int n = 2;
  if (hs.goff[e] >= 0)
    for (int a = 0; a < 3; ++a) n = std::max(n, static_cast<int>(hs.gmodes[3 * e + a]));
  if (hs.foff[e] >= 0)
    for (int a = 0; a < 3; ++a) n = std::max(n, static_cast<int>(hs.fmodes[3 * e + a]));
  return n;
}

// One element's record at n modes per direction into r (record_floats(n)
// zeroed floats); returns the element's flags and own geometry modes.
static uint32_t pack_one(const HostScene& hs, int64_t e, int N, float* r, int32_t& own) {
  const int64_t S = block_floats(N), RS = row_stride(N);
  uint32_t fl = 0;
  if (hs.goff[e] >= 0) {
    const uint32_t mx = hs.gmodes[3 * e], my = hs.gmodes[3 * e + 1], mz = hs.gmodes[3 * e + 2];
    const int64_t cnt = static_cast<int64_t>(mx) * my * mz;
    for (int c = 0; c < 3; ++c) {
      const float* src = hs.geom.data() + hs.goff[e] + c * cnt;
      for (uint32_t k = 0; k < mz; ++k)
        for (uint32_t j = 0; j < my; ++j)
          for (uint32_t i = 0; i < mx; ++i) r[c * S + (k * N + j) * RS + i] = src[(k * my + j) * mx + i];
    }
    own = static_cast<int32_t>(std::max(mx, std::max(my, mz)));
  } else {
    // trilinear map == N=2 modal map with the corners as coefficients
    const float* cv = hs.corners.data() + e * 24;
    for (int v = 0; v < 8; ++v) {
      const int z = kXml2Z[v];
      const int i = z & 1, j = (z >> 1) & 1, k = (z >> 2) & 1;
      for (int c = 0; c < 3; ++c) r[c * S + (k * N + j) * RS + i] = cv[3 * v + c];
    }
    fl |= 2u;
    own = 0;
  }
  if (hs.foff[e] >= 0) {
    const uint32_t mx = hs.fmodes[3 * e], my = hs.fmodes[3 * e + 1], mz = hs.fmodes[3 * e + 2];
    if (mx > 0 && my > 0 && mz > 0) {
      const float* src = hs.field.data() + hs.foff[e];
      for (uint32_t k = 0; k < mz; ++k)
        for (uint32_t j = 0; j < my; ++j)
          for (uint32_t i = 0; i < mx; ++i) r[3 * S + (k * N + j) * RS + i] = src[(k * my + j) * mx + i];
      fl |= 1u;
    }
  }
  return fl;
}

void pack_records(const HostScene& hs, int N, std::vector<float>& rec, std::vector<uint32_t>& flags,
                  std::vector<int32_t>& own) {
  const int64_t ne = hs.size();
  rec.assign(static_cast<size_t>(ne) * record_floats(N), 0.0f);
  flags.assign(ne, 0);
  own.assign(ne, 0);
  parallel_chunks(ne, [&](int64_t b, int64_t e_end) {
    for (int64_t e = b; e < e_end; ++e) flags[e] = pack_one(hs, e, N, rec.data() + e * record_floats(N), own[e]);
  });
}

void pack_compact(const HostScene& hs, std::vector<float>& rec, std::vector<int64_t>& off, std::vector<uint8_t>& order) {
  const int64_t ne = hs.size();
  off.assign(ne, 0);
  order.assign(ne, 0);
  int64_t total = 0;
  for (int64_t e = 0; e < ne; ++e) {
    const int n = element_order(hs, e);
    order[e] = static_cast<uint8_t>(n);
    off[e] = total;
    total += record_floats(n);
  }
  rec.assign(static_cast<size_t>(total), 0.0f);
  parallel_chunks(ne, [&](int64_t b, int64_t e_end) {
    for (int64_t e = b; e < e_end; ++e) {
      int32_t own;
      pack_one(hs, e, order[e], rec.data() + off[e], own);
    }
  });
}

// phi_i(x) = sum_k M[i][k] B_k(s), s = (x-a)/(b-a), B_k = C(p,k) s^k (1-s)^(p-k),
// p = n-1: solve the Bernstein collocation system at n Chebyshev points.
void modal_to_bernstein(int n, double a, double b, std::vector<double>& M) {
  const int p = n - 1;
  std::vector<double> s(n), Bm(static_cast<size_t>(n) * n), Binv;
  for (int r = 0; r < n; ++r) s[r] = n == 1 ? 0.5 : 0.5 - 0.5 * std::cos(M_PI * (r + 0.5) / n);
  for (int r = 0; r < n; ++r) {
    double binom = 1.0;
    for (int k = 0; k <= p; ++k) {
      if (k > 0) binom = binom * (p - k + 1) / k;
      Bm[r * n + k] = binom * std::pow(s[r], k) * std::pow(1.0 - s[r], p - k);
    }
  }
  invert_dense(Bm, n, Binv);
  M.assign(static_cast<size_t>(n) * n, 0.0);
  for (int i = 0; i < n; ++i) {
    // values of phi_i at the collocation points, then solve B c = v
    std::vector<double> v(n);
    for (int r = 0; r < n; ++r) v[r] = mod_a(i, a + (b - a) * s[r]);
    for (int k = 0; k < n; ++k) {
      double acc = 0;
      for (int r = 0; r < n; ++r) acc += Binv[k * n + r] * v[r];
      M[i * n + k] = acc;
    }
  }
}

}  // namespace ho
