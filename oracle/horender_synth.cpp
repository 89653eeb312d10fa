// Seeded synthetic scenes on the CPU side (TEST INFRASTRUCTURE ONLY): the
// scene description that ho_generate_synthetic documents in horender.h,
// computed here without the product library, so the benchmark's CPU arm and
// the tests can build a workload's scene with the oracle alone.
//
// The description: an nx*ny*nz grid of hexes over [0,1]^3; per element n^3
// GLL nodes (n = P + 1), displaced by A*h*sin(2 pi x)sin(2 pi y)sin(2 pi z)
// with the same scalar added to x, y and z; a field of Gaussians (centres
// U[0,1]^3, sigma U[0.1,0.3], amplitude U[-1,1]) sampled at the displaced
// nodes; geometry and field fitted to Modified-A modal coefficients in FP64
// (one inverse-Vandermonde solve per direction) and stored as FP32. Random
// numbers: PCG64 (the XSL-RR 128/64 member of O'Neill's PCG family), stream 1
// for the Gaussians (centre x, y, z, sigma, amplitude per Gaussian), stream 2
// for the per-element orders; uniforms from the top 53 bits.
//
// The arithmetic is written in the same order as the library's generator so
// that, on a host compiler that does not fuse multiply-adds, the FP32
// coefficients come out identical; tests compare the two.
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

extern "C" {
typedef struct {
  int32_t nx, ny, nz;
  int32_t order_min, order_max;
  double curve_amp;
  int32_t n_gauss;
  uint64_t seed;
} hor_synth_params;
}

namespace {

constexpr int kMinN = 2, kMaxN = 9;

struct Pcg {
  unsigned __int128 s = 0, inc = 0;
  Pcg(uint64_t seed, uint64_t stream) {
    inc = (static_cast<unsigned __int128>(stream) << 1) | 1u;
    step();
    s += seed;
    step();
  }
  uint64_t step() {
    static const unsigned __int128 mult =
        (static_cast<unsigned __int128>(0x2360ED051FC65DA4ULL) << 64) | 0x4385DF649FCCF645ULL;
    const unsigned __int128 old = s;
    s = old * mult + inc;
    const uint64_t folded = static_cast<uint64_t>(old >> 64) ^ static_cast<uint64_t>(old);
    const unsigned r = static_cast<unsigned>(old >> 122);
    return (folded >> r) | (folded << ((64u - r) & 63u));
  }
  double u01() { return static_cast<double>(step() >> 11) * (1.0 / 9007199254740992.0); }
};

// Modified-A mode i at x: the two vertex modes, then (1-x^2)/4 times the
// Jacobi polynomial P^{(1,1)}_{i-2} (three-term recurrence).
double mode_a(int i, double x) {
  if (i == 0) return 0.5 * (1.0 - x);
  if (i == 1) return 0.5 * (1.0 + x);
  const int m = i - 2;
  double p0 = 1.0, p1 = 2.0 * x;
  double p = m == 0 ? p0 : p1;
  for (int k = 2; k <= m; ++k) {
    const double a = double((2 * k + 1) * (k + 1)) / double(k * (k + 2));
    const double b = double(k + 1) / double(k + 2);
    p = a * x * p1 - b * p0;
    p0 = p1;
    p1 = p;
  }
  return 0.25 * (1.0 - x * x) * p;
}

// Legendre P_N(x) and its derivative.
void legendre_pd(int N, double x, double& p, double& dp) {
  if (N == 0) {
    p = 1.0;
    dp = 0.0;
    return;
  }
  double a = 1.0, b = x;
  for (int k = 2; k <= N; ++k) {
    const double c = ((2.0 * k - 1.0) * x * b - (k - 1.0) * a) / k;
    a = b;
    b = c;
  }
  p = b;
  dp = N * (x * b - a) / (x * x - 1.0);
}

// Gauss-Lobatto-Legendre nodes: the ends and the roots of P'_{n-1}, by
// Newton from the Chebyshev-Lobatto points, then made exactly antisymmetric.
std::vector<double> lobatto(int n) {
  std::vector<double> x(n, 0.0);
  if (n == 1) return x;
  const int N = n - 1;
  x[0] = -1.0;
  x[N] = 1.0;
  for (int i = 1; i < N; ++i) {
    double t = -std::cos(M_PI * i / N);
    for (int it = 0; it < 100; ++it) {
      double p, dp;
      legendre_pd(N, t, p, dp);
      const double d2 = (2.0 * t * dp - N * (N + 1.0) * p) / (1.0 - t * t);
      const double dt = dp / d2;
      t -= dt;
      if (std::fabs(dt) < 1e-16) break;
    }
    x[i] = t;
  }
  for (int i = 0; i < n / 2; ++i) {
    const double h = 0.5 * (x[n - 1 - i] - x[i]);
    x[i] = -h;
    x[n - 1 - i] = h;
  }
  if (n % 2) x[n / 2] = 0.0;
  return x;
}

// Inverse of V[r][c] = mode_a(c, node r) by Gauss-Jordan elimination with
// partial pivoting.
bool vinv_of(const std::vector<double>& nodes, std::vector<double>& inv) {
  const int n = static_cast<int>(nodes.size());
  std::vector<double> a(static_cast<size_t>(n) * n);
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) a[r * n + c] = mode_a(c, nodes[r]);
  inv.assign(static_cast<size_t>(n) * n, 0.0);
  for (int i = 0; i < n; ++i) inv[i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int pr = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(a[r * n + c]) > std::fabs(a[pr * n + c])) pr = r;
    if (std::fabs(a[pr * n + c]) < 1e-300) return false;
    if (pr != c)
      for (int k = 0; k < n; ++k) {
        std::swap(a[c * n + k], a[pr * n + k]);
        std::swap(inv[c * n + k], inv[pr * n + k]);
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

// modal = (Vinv x Vinv x Vinv) nodal, first direction first.
void fit3(int n, const std::vector<double>& vi, const double* nodal, double* t1, double* t2, float* out) {
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int a = 0; a < n; ++a) {
        double s = 0;
        for (int i = 0; i < n; ++i) s += vi[a * n + i] * nodal[(k * n + j) * n + i];
        t1[(k * n + j) * n + a] = s;
      }
  for (int k = 0; k < n; ++k)
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a) {
        double s = 0;
        for (int j = 0; j < n; ++j) s += vi[b * n + j] * t1[(k * n + j) * n + a];
        t2[(k * n + b) * n + a] = s;
      }
  for (int c = 0; c < n; ++c)
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a) {
        double s = 0;
        for (int k = 0; k < n; ++k) s += vi[c * n + k] * t2[(k * n + b) * n + a];
        out[(c * n + b) * n + a] = static_cast<float>(s);
      }
}

bool valid(const hor_synth_params* p) {
  return p && p->nx > 0 && p->ny > 0 && p->nz > 0 && p->order_min >= kMinN - 1 && p->order_max <= kMaxN - 1 &&
         p->order_min <= p->order_max && p->n_gauss >= 0;
}

std::vector<int> element_orders(const hor_synth_params& p) {
  const int64_t ne = static_cast<int64_t>(p.nx) * p.ny * p.nz;
  std::vector<int> order(ne, p.order_min);
  if (p.order_max > p.order_min) {
    Pcg r(p.seed, 2);
    const int span = p.order_max - p.order_min + 1;
    for (int64_t e = 0; e < ne; ++e) {
      const int k = static_cast<int>(r.u01() * span);
      order[e] = p.order_min + (k < span - 1 ? k : span - 1);
    }
  }
  return order;
}

}  // namespace

extern "C" {

// Sizes of the scene: elements, geometry floats, field floats.
int hor_synth_sizes(const hor_synth_params* p, int64_t* n_elem, int64_t* geom_len, int64_t* field_len) {
  if (!valid(p)) return -1;
  const std::vector<int> order = element_orders(*p);
  int64_t g = 0, f = 0;
  for (int o : order) {
    const int64_t S = static_cast<int64_t>(o + 1) * (o + 1) * (o + 1);
    g += 3 * S;
    f += S;
  }
  *n_elem = static_cast<int64_t>(order.size());
  *geom_len = g;
  *field_len = f;
  return 0;
}

// Fills the arrays hor_synth_sizes sized: corners n*8*3 (XML vertex order),
// modes n*3 (geometry and field alike), offsets n (x block, then y, z), the
// coefficient pools. nthreads <= 0: all hardware threads.
int hor_synth_fill(const hor_synth_params* p, int nthreads, float* verts, uint32_t* geom_modes,
                   int64_t* geom_offset, float* geom, uint32_t* field_modes, int64_t* field_offset, float* field) {
  if (!valid(p)) return -1;
  const hor_synth_params P = *p;
  Pcg rg(P.seed, 1);
  std::vector<double> gx(P.n_gauss), gy(P.n_gauss), gz(P.n_gauss), gsig(P.n_gauss), gamp(P.n_gauss);
  for (int g = 0; g < P.n_gauss; ++g) {
    gx[g] = rg.u01();
    gy[g] = rg.u01();
    gz[g] = rg.u01();
    gsig[g] = 0.1 + 0.2 * rg.u01();
    gamp[g] = -1.0 + 2.0 * rg.u01();
  }
  const std::vector<int> order = element_orders(P);
  const int64_t ne = static_cast<int64_t>(order.size());
  int64_t go = 0, fo = 0;
  for (int64_t e = 0; e < ne; ++e) {
    const int n = order[e] + 1;
    const int64_t S = static_cast<int64_t>(n) * n * n;
    geom_offset[e] = go;
    field_offset[e] = fo;
    go += 3 * S;
    fo += S;
    for (int a = 0; a < 3; ++a) {
      geom_modes[3 * e + a] = static_cast<uint32_t>(n);
      field_modes[3 * e + a] = static_cast<uint32_t>(n);
    }
  }
  std::vector<std::vector<double>> nodes(kMaxN + 1), vi(kMaxN + 1);
  for (int n = kMinN; n <= kMaxN; ++n) {
    nodes[n] = lobatto(n);
    if (!vinv_of(nodes[n], vi[n])) return -2;
  }
  const double hx = 1.0 / P.nx, hy = 1.0 / P.ny, hz = 1.0 / P.nz;
  const double h = std::fmin(hx, std::fmin(hy, hz));
  const double amp = P.curve_amp * h;
  const double tau = 2.0 * M_PI;
  auto bump = [&](double x, double y, double z) {
    return amp * std::sin(tau * x) * std::sin(tau * y) * std::sin(tau * z);
  };
  auto one = [&](int64_t e, std::vector<double>& buf) {
    const int kx = static_cast<int>(e % P.nx), ky = static_cast<int>((e / P.nx) % P.ny),
              kz = static_cast<int>(e / (static_cast<int64_t>(P.nx) * P.ny));
    const int n = order[e] + 1;
    const int S = n * n * n;
    const std::vector<double>& r = nodes[n];
    double* X = buf.data();
    double* Y = X + S;
    double* Z = Y + S;
    double* U = Z + S;
    double* t1 = U + S;
    double* t2 = t1 + S;
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const double x0 = (kx + 0.5 * (r[i] + 1.0)) * hx;
          const double y0 = (ky + 0.5 * (r[j] + 1.0)) * hy;
          const double z0 = (kz + 0.5 * (r[k] + 1.0)) * hz;
          const double dl = bump(x0, y0, z0);
          const double x = x0 + dl, y = y0 + dl, z = z0 + dl;
          double u = 0.0;
          for (int g = 0; g < P.n_gauss; ++g) {
            const double dx = x - gx[g], dy = y - gy[g], dz = z - gz[g];
            u += gamp[g] * std::exp(-(dx * dx + dy * dy + dz * dz) / (2.0 * gsig[g] * gsig[g]));
          }
          const int q = (k * n + j) * n + i;
          X[q] = x;
          Y[q] = y;
          Z[q] = z;
          U[q] = u;
        }
    float* gd = geom + geom_offset[e];
    for (int c = 0; c < 3; ++c) fit3(n, vi[n], X + c * S, t1, t2, gd + c * S);
    fit3(n, vi[n], U, t1, t2, field + field_offset[e]);
    static const int cx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cy[8] = {0, 0, 1, 1, 0, 0, 1, 1},
                     cz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    float* v = verts + 24 * e;
    for (int c = 0; c < 8; ++c) {
      const double x0 = (kx + cx[c]) * hx, y0 = (ky + cy[c]) * hy, z0 = (kz + cz[c]) * hz;
      const double dl = bump(x0, y0, z0);
      v[3 * c] = static_cast<float>(x0 + dl);
      v[3 * c + 1] = static_cast<float>(y0 + dl);
      v[3 * c + 2] = static_cast<float>(z0 + dl);
    }
  };
  int nt = nthreads > 0 ? nthreads : static_cast<int>(std::thread::hardware_concurrency());
  if (nt < 1) nt = 1;
  std::atomic<int64_t> next{0};
  auto worker = [&] {
    std::vector<double> buf(6 * kMaxN * kMaxN * kMaxN);
    for (;;) {
      const int64_t b = next.fetch_add(64);
      if (b >= ne) break;
      const int64_t end = b + 64 < ne ? b + 64 : ne;
      for (int64_t e = b; e < end; ++e) one(e, buf);
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
  worker();
  for (auto& th : pool) th.join();
  return 0;
}

}  // extern "C"
