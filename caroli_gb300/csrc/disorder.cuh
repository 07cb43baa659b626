// On-device disorder: the H values of many configurations generated on the GPU from the clean
// values and the CLI's [[disorder]] entries (caroli-cli/src/build.rs:251-310), bit for bit the
// host's (caroli-disorder/src/{rng,lib}.rs):
//   - xoshiro256** seeded by splitmix64 (rng.rs:9-33), uniform = top 53 bits (rng.rs:65-69),
//     integer(lo, hi) = lo + floor((hi - lo + 1) u);
//   - Anderson: w (u - 1/2) per site in region order (lib.rs:110-115);
//   - magnetic impurities: partial Fisher-Yates choice of floor(c N) sites (lib.rs:14-26), then all
//     n_z draws, then all azimuths (lib.rs:53-64); J (n_x S_x + n_y S_y + n_z S_z) on each
//     (lib.rs:88-100), summed in that order.
// Every product and sum is rounded on its own (__dmul_rn / __dadd_rn), as the host evaluates
// them, so the values match the host's exactly; only the azimuth's cos and sin (isotropic and cone
// moments) may differ from the host's libm in the last bit.
#pragma once
#include <cstdint>

namespace caroli {

enum { DIS_ANDERSON = 0, DIS_MAGNETIC = 1 };
enum { MOM_ISOTROPIC = 0, MOM_POLARIZED = 1, MOM_CONE = 2 };

struct DisorderDev {
  int32_t kind, moments;
  uint64_t seed;
  double strength, exchange, mparam;  // mparam: mz (polarized) or -(1 - cos θ0) (cone)
  int32_t n_imp, orb;                 // impurities per configuration; orbitals of a site (magnetic)
  const double2* spin;                // S_x, S_y, S_z: orb x orb column-major each
};

struct Xoshiro {
  uint64_t s[4];
  __device__ static uint64_t splitmix(uint64_t& st) {
    st += 0x9E3779B97F4A7C15ull;
    uint64_t z = st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  __device__ explicit Xoshiro(uint64_t seed) {
    uint64_t st = seed;
    for (int k = 0; k < 4; ++k) s[k] = splitmix(st);
  }
  __device__ static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  __device__ uint64_t next() {
    const uint64_t result = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return result;
  }
  __device__ double uniform() { return __dmul_rn((double)(next() >> 11), 1.0 / 9007199254740992.0); }
  __device__ int64_t integer(int64_t lo, int64_t hi) {
    return lo + (int64_t)__dmul_rn((double)(hi - lo + 1), uniform());
  }
};

// One thread per (entry, configuration): the entry's draws for configuration first + c, in the
// host's order. Anderson: scal[e][c][site]. Magnetic: coef[e][c][site] = (J n_x, J n_y, J n_z) and
// flag = 1 on the chosen sites; tab is a scratch permutation of nsites per (entry, configuration).
__global__ void disorder_draw_kernel(const DisorderDev* __restrict__ ent, int nent, int nconf, int first, int nsites,
                                     double* __restrict__ scal, double* __restrict__ coef,
                                     uint8_t* __restrict__ flag, int32_t* __restrict__ tab) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nent * nconf) return;
  const int e = t / nconf, c = t % nconf;
  const DisorderDev& d = ent[e];
  Xoshiro rng(d.seed + (uint64_t)(first + c));
  const size_t base = ((size_t)e * nconf + c) * (size_t)nsites;
  if (d.kind == DIS_ANDERSON) {
    for (int i = 0; i < nsites; ++i) scal[base + i] = __dmul_rn(d.strength, __dsub_rn(rng.uniform(), 0.5));
    return;
  }
  int32_t* tb = tab + base;
  for (int i = 0; i < nsites; ++i) {
    tb[i] = i;
    flag[base + i] = 0;
  }
  for (int i = 0; i < d.n_imp; ++i) {
    const int r = (int)rng.integer(i + 1, nsites) - 1;
    const int32_t a = tb[i];
    tb[i] = tb[r];
    tb[r] = a;
  }
  // n_z of every impurity, then every azimuth (kept in coef until both are drawn).
  for (int i = 0; i < d.n_imp; ++i) {
    const double u = rng.uniform();
    double nz;
    if (d.moments == MOM_ISOTROPIC) nz = __dsub_rn(__dmul_rn(2.0, u), 1.0);
    else if (d.moments == MOM_CONE) nz = __dadd_rn(__dmul_rn(d.mparam, u), 1.0);
    else nz = __dsub_rn(__dadd_rn(__dmul_rn(__dmul_rn(2.0, __dsub_rn(1.0, d.mparam)), u), __dmul_rn(2.0, d.mparam)), 1.0);
    coef[(base + tb[i]) * 3 + 2] = nz;
  }
  const double two_pi = 6.283185307179586;  // 2.0 * pi in double, as the host multiplies
  for (int i = 0; i < d.n_imp; ++i) {
    const double phi = __dmul_rn(two_pi, rng.uniform());
    const size_t k = (base + tb[i]) * 3;
    const double z = coef[k + 2];
    const double perp = __dsqrt_rn(__dsub_rn(1.0, __dmul_rn(z, z)));
    const double nx = __dmul_rn(perp, cos(phi)), ny = __dmul_rn(perp, sin(phi));
    coef[k] = __dmul_rn(d.exchange, nx);
    coef[k + 1] = __dmul_rn(d.exchange, ny);
    coef[k + 2] = __dmul_rn(d.exchange, z);
    flag[base + tb[i]] = 1;
  }
}

// Values of configuration c: the clean value of every stored entry plus, on the on-site blocks,
// each entry's term in order. grid (nnz chunks, configurations).
__global__ void __launch_bounds__(256) disorder_apply_kernel(const DisorderDev* __restrict__ ent, int nent, int nconf,
                                                             int nsites, int64_t nnz, const double2* __restrict__ clean,
                                                             const int32_t* __restrict__ os_site,
                                                             const int16_t* __restrict__ os_ab,
                                                             const double* __restrict__ scal,
                                                             const double* __restrict__ coef,
                                                             const uint8_t* __restrict__ flag, double2* __restrict__ out) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (q >= nnz) return;
  double2 v = clean[q];
  const int site = os_site[q];
  if (site >= 0) {
    const int a = os_ab[2 * q], b = os_ab[2 * q + 1];
    for (int e = 0; e < nent; ++e) {
      const DisorderDev& d = ent[e];
      const size_t at = ((size_t)e * nconf + c) * (size_t)nsites + site;
      if (d.kind == DIS_ANDERSON) {
        if (a == b) v.x = __dadd_rn(v.x, scal[at]);
      } else if (flag[at]) {
        const double* k = coef + at * 3;
        const int64_t m = a + (int64_t)b * d.orb, sz = (int64_t)d.orb * d.orb;
        double re = 0.0, im = 0.0;
        for (int s = 0; s < 3; ++s) {
          const double2 sv = d.spin[s * sz + m];
          re = __dadd_rn(re, __dmul_rn(k[s], sv.x));
          im = __dadd_rn(im, __dmul_rn(k[s], sv.y));
        }
        v.x = __dadd_rn(v.x, re);
        v.y = __dadd_rn(v.y, im);
      }
    }
  }
  out[(size_t)c * nnz + q] = v;
}

}  // namespace caroli
