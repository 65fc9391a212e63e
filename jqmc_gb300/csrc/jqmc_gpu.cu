// libjqmc_gpu: the jQMC walker hot path on one GB300 (sm_103a).
//
// One CTA owns one walker.  The basis / ECP tables are staged into shared
// memory at kernel start; the per-walker ratio tables T_up, T_dn and the J3
// field live in HBM and are read through L1.  Threads split a walker's work by
// mesh point (kinetic lattice moves, ECP quadrature points), by electron, or by
// AO index, and every thread walks the shell list in the same order, so the
// AO loops are branch-uniform across a warp.
//
// Algebra (n = N_up = N_dn, A = number of geminal AOs, lambda the AO pairing
// matrix, Phi the AO tables at the electrons, G = Phi_up^T lambda Phi_dn):
//   T_up = lambda Phi_dn G^-1   (row i: up electron i),
//   T_dn = G^-1 Phi_up^T lambda (row j: dn electron j).
// Moving up electron i to r' multiplies det G by phi(r') . T_up[i]; moving dn
// electron j by T_dn[j] . phi(r').  grad_i ln det = grad phi(r_i) . T_up[i] and
// lap_i ln det = lap phi(r_i) . T_up[i] - |grad_i ln det|^2.  After a move the
// tables are patched by rank-1 (Sherman-Morrison) updates plus one lambda
// mat-vec; see sm_move below.
//
// J3 = j1 . sum_e phi3_e + sum_{pairs} phi3_a^T J phi3_b is linear in each
// electron's J3-AO vector, so the field h_e = dJ3/dphi3_e gives
// Delta J3 = (phi3(r') - phi3(r_e)) . h_e, grad_e J3 = grad phi3(r_e) . h_e and
// lap_e J3 = lap phi3(r_e) . h_e.
//
// Two forms share this code through templates:
//   plain FP64 (JQMC_PREC_FP64): every quantity in double;
//   mixed      (JQMC_PREC_MIXED): AO values, ratios, T tables, G^-1, the J3
//     field and the Sherman-Morrison updates in float (exp on the SFU); the
//     continuum kinetic energy (AO gradients/Laplacians), every energy and
//     weight accumulation, and the rebuild of the tables from the positions
//     (jqmc_walker_init) in double.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <type_traits>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "jqmc_gpu.h"
#include "jqmc_tc.h"
#include "solid_harmonics.cuh"

namespace {

// Threads per CTA of the LRDMC kernels (one walker per CTA) and the CTAs per SM
// their register budget is sized for.  The float projection runs 8 warps per
// walker at 2 CTAs per SM (16 warps per SM; 12 % faster on the chain than 4
// warps at 3 CTAs); the FP64 and block-energy kernels keep 4 warps at 3 CTAs
// (170 registers, which their FP64 paths need).
template <class R, class Acc>
struct LrdmcShape {
  static constexpr int threads = 128, min_ctas = 3;
};
template <>
struct LrdmcShape<float, float> {
  static constexpr int threads = 256, min_ctas = 2;
};

constexpr int kSlots = JQMC_ECP_SLOTS;
constexpr int kRed = 64;  // doubles of reduction scratch

// Per-electron energy cache (double): quantities that depend on one electron's
// position, or on its pairs, kept current by every move instead of being
// recomputed each step.  Row e (kEC doubles) per electron, then one row of
// walker totals.
constexpr int kEC = JQMC_ECACHE_STRIDE;
enum {
  EC_EI = 0,     // electron-ion Coulomb of electron e
  EC_ELOC = 1,   // local ECP channel of electron e, summed over nuclei
  EC_J1G = 2,    // grad J1 (3)
  EC_J1L = 5,    // lap J1
  EC_J2G = 6,    // grad J2 (3)
  EC_J2L = 9,    // lap J2
  EC_NEAR = 10,  // nearest nucleus (as double)
  EC_DIST = 11,  // distance to it
  EC_VL = 12,    // non-local channel values V_l at the nearest nucleus (kSlots)
  EC_TOT_EE = 0  // totals row: e-e Coulomb
};
static_assert(EC_VL + kSlots <= kEC, "energy cache row too short");

template <class R>
struct Num;
template <>
struct Num<double> {
  static __device__ __forceinline__ double ex(double x) { return exp(x); }
  static __device__ __forceinline__ double sq(double x) { return sqrt(x); }
  static __device__ __forceinline__ double em1(double x) { return expm1(x); }
};
template <>
struct Num<float> {
  static __device__ __forceinline__ float ex(float x) { return __expf(x); }
  static __device__ __forceinline__ float sq(float x) { return sqrtf(x); }
  static __device__ __forceinline__ float em1(float x) { return expm1f(x); }
};

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Ask L2 for the 128-byte lines of [p, p + bytes), one line per lane (bounded
// to the given range; a hint only, no data is returned).
__device__ __forceinline__ void prefetch_l2(const void* p, size_t bytes, int lane) {
  const char* c = static_cast<const char*>(p);
  for (size_t off = (size_t)lane * 128; off < bytes; off += 32 * 128)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(c + off));
}

// Accumulators of the mesh and electron-term sums.  float / double: plain
// sums.  F2: compensated float-float sum of float products (TwoProduct by FMA
// and TwoSum, as in algorithm Dot2 of Ogita, Rump and Oishi, SIAM J. Sci.
// Comput. 26 (2005) 1955-1988): FP32-pipe work with the cancellation error of
// a double sum.  acc_out() reduces over the warp (every lane gets the result):
// float for float, double for double and F2.
struct F2 {
  float s, c;
  float m;   // sum of |terms| (the scale of the rounding of the float inputs)
};
// the block energy of the mixed form, like the float projection, at 8 warps per
// walker and 2 CTAs per SM (11 % faster than 4 warps at 3 CTAs on the chain)
template <>
struct LrdmcShape<float, F2> {
  static constexpr int threads = 256, min_ctas = 2;
};
__device__ __forceinline__ void acc_zero(float& a) { a = 0.f; }
__device__ __forceinline__ void acc_zero(double& a) { a = 0.0; }
__device__ __forceinline__ void acc_zero(F2& a) { a.s = 0.f; a.c = 0.f; a.m = 0.f; }
// sums of |terms| (compensated accumulators only)
__device__ __forceinline__ void acc_mag(F2& a, float v) { a.m += v; }
__device__ __forceinline__ float acc_mag_out(F2 a) { return warp_sum(a.m); }
__device__ __forceinline__ void acc_fma(float& a, float x, float y) { a += x * y; }
__device__ __forceinline__ void acc_fma(double& a, double x, double y) { a += x * y; }
__device__ __forceinline__ void two_sum_into(F2& a, float p) {
  const float t = __fadd_rn(a.s, p);
  const float z = __fsub_rn(t, a.s);
  a.c += __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, z)), __fsub_rn(p, z));
  a.s = t;
}
__device__ __forceinline__ void acc_fma(F2& a, float x, float y) {
  const float p = __fmul_rn(x, y);
  a.c += __fmaf_rn(x, y, -p);
  two_sum_into(a, p);
}
__device__ __forceinline__ void acc_add(float& a, float x) { a += x; }
__device__ __forceinline__ void acc_add(double& a, double x) { a += x; }
__device__ __forceinline__ void acc_add(F2& a, float x) { two_sum_into(a, x); }
__device__ __forceinline__ float acc_out(float a) { return warp_sum(a); }
__device__ __forceinline__ double acc_out(double a) { return warp_sum(a); }
__device__ __forceinline__ double acc_out(F2 a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float s2 = __shfl_xor_sync(0xffffffffu, a.s, o);
    const float c2 = __shfl_xor_sync(0xffffffffu, a.c, o);
    a.c += c2;
    two_sum_into(a, s2);
  }
  return (double)a.s + (double)a.c;
}
template <class A> struct AccTraits { using out = A; using arith = A; static constexpr bool accurate = false; };
template <> struct AccTraits<F2> { using out = double; using arith = float; static constexpr bool accurate = true; };
// exponentials of the mesh: the fast intrinsic in the float projection, the
// correctly rounded-to-1-ulp expf / expm1f where the sums are compensated
template <class R, bool ACC>
struct MeshExp {
  static __device__ __forceinline__ R ex(R x) { return Num<R>::ex(x); }
  static __device__ __forceinline__ R em1(R x) { return Num<R>::em1(x); }
};
template <>
struct MeshExp<float, true> {
  static __device__ __forceinline__ float ex(float x) { return expf(x); }
  static __device__ __forceinline__ float em1(float x) { return expm1f(x); }
};

// Device shell records: the 8 ints of jqmc_basis_desc, then the square of the
// shell's reach radius as float bits (field 8), so that lanes reading one field
// of consecutive shells hit distinct shared-memory banks (a stride of 9 words is
// coprime with the 32 banks).  Beyond its reach radius from the shell's nucleus,
// every AO of the shell is below e^-kReach in magnitude for unit table entries:
// sum_q |c_q| max(r, 1)^l e^(-Z_q r^2).
constexpr int kSh = 9;
constexpr int kShReach = 8;
constexpr double kReach = 40.0;

struct Basis {
  int nshell, nao, nprim;
  const int* shells;
  const double* prims;   // (Z, cN) double
  const float* primsf;   // (Z, cN) float copy
};

template <class R>
__device__ __forceinline__ const R* prims_of(const Basis& b);
template <>
__device__ __forceinline__ const double* prims_of<double>(const Basis& b) { return b.prims; }
template <>
__device__ __forceinline__ const float* prims_of<float>(const Basis& b) { return b.primsf; }

struct Sys {
  int natom, n_up, n_dn, N;
  const double* atom_pos;
  const double* atom_zeff;
  Basis det;
  const double* lam;   // A x A row-major
  const double* lamT;  // transpose
  const float* lamf;
  const float* lamTf;
  const float* laml;   // lam - (double)lamf: the low float of a float-float split
  const float* lamTl;
  int has_j1, j1_type;
  double j1_param;
  const double* j1_cA;   // natom x 2: ((2Z)^(1/4), (2Z)^(3/4)) with Z the J1 effective charge
  int has_j2, j2_type;
  double j2_param;
  int has_j3;
  Basis j3;
  const double* j3mat;   // A3 x A3
  const double* j3matT;  // transpose
  const double* j3vec;   // A3
  const float* j3matf;
  const float* j3matTf;
  const float4* j3k4;   // (cp, c): float pairs of J[cp][c] and J[c][cp] (hi, lo, hi, lo)
  int ecp_flag;
  const int* ecp_maxl1;
  const int* ecp_chan;
  int ecp_nterm;
  const double* ecp_terms;
  int nv;
  const double* mesh_pts;
  const double* mesh_w;
  double ion_ion;
  int dlt;   // LRDMC non-local moves: 0 T-move, 1 determinant locality (dltmove)
};

template <class T>
__device__ __forceinline__ const T* lam_of(const Sys& s);
template <>
__device__ __forceinline__ const double* lam_of<double>(const Sys& s) { return s.lam; }
template <>
__device__ __forceinline__ const float* lam_of<float>(const Sys& s) { return s.lamf; }
template <class T>
__device__ __forceinline__ const T* lamT_of(const Sys& s);
template <>
__device__ __forceinline__ const double* lamT_of<double>(const Sys& s) { return s.lamT; }
template <>
__device__ __forceinline__ const float* lamT_of<float>(const Sys& s) { return s.lamTf; }
template <class T>
__device__ __forceinline__ const T* j3m_of(const Sys& s);
template <>
__device__ __forceinline__ const double* j3m_of<double>(const Sys& s) { return s.j3mat; }
template <>
__device__ __forceinline__ const float* j3m_of<float>(const Sys& s) { return s.j3matf; }
template <class T>
__device__ __forceinline__ const T* j3mT_of(const Sys& s);
template <>
__device__ __forceinline__ const double* j3mT_of<double>(const Sys& s) { return s.j3matT; }
template <>
__device__ __forceinline__ const float* j3mT_of<float>(const Sys& s) { return s.j3matTf; }

// Device view of a jqmc_walkers descriptor (tables typed at the kernel).
struct WS {
  double* r;
  void *G, *Ginv, *Tup, *Tdn, *h3, *dphi, *dphi3;
  double* ecache;
  float* dcache;
  double* scratch;
  int* status;
  float* tlo;   // mixed form, optional: low parts of the FP64-accurate T tables
};

// Shared-memory table layout (byte offsets), identical for every walker kernel.
struct TableLayout {
  int off_dsh, off_dpr, off_dprf, off_jsh, off_jpr, off_jprf, off_apos, off_azeff, off_j1z, off_maxl1, off_chan, off_terms,
      off_mpts, off_mw;
  int f64prims;   // stage the double primitive tables (the float kernels read them from L1/L2)
  int bytes;
};

__host__ __device__ inline int align16(int x) { return (x + 15) & ~15; }

// Floats per walker of the low-part buffer (jqmc_walkers.tlo): T_up and T_dn
// rows, then the J3 field's N rows.
__host__ __device__ inline size_t tlo_stride(const Sys& s) {
  return (size_t)2 * s.n_up * s.det.nao + (s.has_j3 ? (size_t)s.N * s.j3.nao : 0);
}

TableLayout table_layout(const Sys& s, bool f64prims = true) {
  TableLayout L;
  int o = 0;
  const int jsh = s.has_j3 ? s.j3.nshell : 0, jpr = s.has_j3 ? s.j3.nprim : 0;
  L.f64prims = f64prims ? 1 : 0;
  L.off_dsh = o; o = align16(o + s.det.nshell * kSh * 4);
  L.off_dpr = o; o = align16(o + (f64prims ? s.det.nprim * 2 * 8 : 0));
  L.off_dprf = o; o = align16(o + s.det.nprim * 2 * 4);
  L.off_jsh = o; o = align16(o + jsh * kSh * 4);
  L.off_jpr = o; o = align16(o + (f64prims ? jpr * 2 * 8 : 0));
  L.off_jprf = o; o = align16(o + jpr * 2 * 4);
  L.off_apos = o; o = align16(o + s.natom * 3 * 8);
  L.off_azeff = o; o = align16(o + s.natom * 8);
  L.off_j1z = o; o = align16(o + s.natom * 16);
  L.off_maxl1 = o; o = align16(o + s.natom * 4);
  L.off_chan = o; o = align16(o + s.natom * kSlots * 2 * 4);
  L.off_terms = o; o = align16(o + s.ecp_nterm * 3 * 8);
  L.off_mpts = o; o = align16(o + s.nv * 3 * 8);
  L.off_mw = o; o = align16(o + s.nv * 8);
  L.bytes = o;
  return L;
}

__device__ void copy_words(void* dst, const void* src, int bytes) {
  if (!src || bytes <= 0) return;
  const int nw = bytes / 4;
  const uint32_t* s = static_cast<const uint32_t*>(src);
  uint32_t* d = static_cast<uint32_t*>(dst);
  for (int k = threadIdx.x; k < nw; k += blockDim.x) d[k] = s[k];
}

// Copy the tables into shared memory and return a Sys whose table pointers
// refer to the shared copies.  Ends with __syncthreads().
__device__ Sys stage_tables(const Sys& g, const TableLayout& L, unsigned char* smem) {
  Sys s = g;
  copy_words(smem + L.off_dsh, g.det.shells, g.det.nshell * kSh * 4);
  copy_words(smem + L.off_dprf, g.det.primsf, g.det.nprim * 8);
  s.det.shells = reinterpret_cast<const int*>(smem + L.off_dsh);
  s.det.primsf = reinterpret_cast<const float*>(smem + L.off_dprf);
  if (L.f64prims) {
    copy_words(smem + L.off_dpr, g.det.prims, g.det.nprim * 16);
    s.det.prims = reinterpret_cast<const double*>(smem + L.off_dpr);
  }
  if (g.has_j3) {
    copy_words(smem + L.off_jsh, g.j3.shells, g.j3.nshell * kSh * 4);
    copy_words(smem + L.off_jprf, g.j3.primsf, g.j3.nprim * 8);
    s.j3.shells = reinterpret_cast<const int*>(smem + L.off_jsh);
    s.j3.primsf = reinterpret_cast<const float*>(smem + L.off_jprf);
    if (L.f64prims) {
      copy_words(smem + L.off_jpr, g.j3.prims, g.j3.nprim * 16);
      s.j3.prims = reinterpret_cast<const double*>(smem + L.off_jpr);
    }
  }
  copy_words(smem + L.off_apos, g.atom_pos, g.natom * 24);
  copy_words(smem + L.off_azeff, g.atom_zeff, g.natom * 8);
  copy_words(smem + L.off_j1z, g.j1_cA, g.natom * 16);
  copy_words(smem + L.off_maxl1, g.ecp_maxl1, g.natom * 4);
  copy_words(smem + L.off_chan, g.ecp_chan, g.natom * kSlots * 8);
  copy_words(smem + L.off_terms, g.ecp_terms, g.ecp_nterm * 24);
  copy_words(smem + L.off_mpts, g.mesh_pts, g.nv * 24);
  copy_words(smem + L.off_mw, g.mesh_w, g.nv * 8);
  s.atom_pos = reinterpret_cast<const double*>(smem + L.off_apos);
  s.atom_zeff = reinterpret_cast<const double*>(smem + L.off_azeff);
  s.j1_cA = reinterpret_cast<const double*>(smem + L.off_j1z);
  s.ecp_maxl1 = reinterpret_cast<const int*>(smem + L.off_maxl1);
  s.ecp_chan = reinterpret_cast<const int*>(smem + L.off_chan);
  s.ecp_terms = reinterpret_cast<const double*>(smem + L.off_terms);
  s.mesh_pts = reinterpret_cast<const double*>(smem + L.off_mpts);
  s.mesh_w = reinterpret_cast<const double*>(smem + L.off_mw);
  __syncthreads();
  return s;
}

// ------------------------------------------------------------------ AO shells
template <int L, class R>
__device__ __forceinline__ void sh_val(R x, R y, R z, R* S) {
  if constexpr (L == 0) sh_l0(x, y, z, S);
  else if constexpr (L == 1) sh_l1(x, y, z, S);
  else if constexpr (L == 2) sh_l2(x, y, z, S);
  else if constexpr (L == 3) sh_l3(x, y, z, S);
  else if constexpr (L == 4) sh_l4(x, y, z, S);
  else if constexpr (L == 5) sh_l5(x, y, z, S);
  else sh_l6(x, y, z, S);
}

template <int L, class R>
__device__ __forceinline__ void sh_grad(R x, R y, R z, R* S, R* G) {
  if constexpr (L == 0) shg_l0(x, y, z, S, G);
  else if constexpr (L == 1) shg_l1(x, y, z, S, G);
  else if constexpr (L == 2) shg_l2(x, y, z, S, G);
  else if constexpr (L == 3) shg_l3(x, y, z, S, G);
  else if constexpr (L == 4) shg_l4(x, y, z, S, G);
  else if constexpr (L == 5) shg_l5(x, y, z, S, G);
  else shg_l6(x, y, z, S, G);
}

template <int L, class R, class F>
__device__ __forceinline__ void emit_val(R dx, R dy, R dz, R rad, int ao0, int jlo, int nm, F& f) {
  R S[2 * L + 1];
  sh_val<L, R>(dx, dy, dz, S);
#pragma unroll
  for (int j = 0; j < 2 * L + 1; ++j) {
    const int k = j - jlo;
    if (k >= 0 && k < nm) f(ao0 + k, rad * S[j]);
  }
}

// value, gradient, Laplacian of every AO of one shell:
//   phi = rad S, grad phi = rad grad S - 2 radZ S d, lap phi = S (4 r^2 radZ2 - (4l+6) radZ)
// (rad = sum_p cN_p e^{-Z_p r^2}, radZ = sum cN Z e, radZ2 = sum cN Z^2 e; the
// solid harmonics are harmonic and homogeneous of degree l).
template <int L, class R, class F>
__device__ __forceinline__ void emit_vgl(R dx, R dy, R dz, R r2, R rad, R radZ, R radZ2, int ao0, int jlo, int nm, F& f) {
  R S[2 * L + 1], G[3 * (2 * L + 1)];
  sh_grad<L, R>(dx, dy, dz, S, G);
  const R lapf = R(4) * r2 * radZ2 - (R(4 * L) + R(6)) * radZ;
#pragma unroll
  for (int j = 0; j < 2 * L + 1; ++j) {
    const int k = j - jlo;
    if (k >= 0 && k < nm) {
      const R t = R(-2) * radZ * S[j];
      f(ao0 + k, rad * S[j], rad * G[3 * j] + t * dx, rad * G[3 * j + 1] + t * dy, rad * G[3 * j + 2] + t * dz,
        S[j] * lapf);
    }
  }
}

// Cartesian shells hold one AO, x^nx y^ny z^nz times the contracted Gaussian:
// component sh[6] - kCartBase of the (l+1)(l+2)/2 in TREXIO order (nx from l
// down, then ny from l - nx down; itertools.combinations_with_replacement).  The
// device shell rows carry the Cartesian kind in field 6 (component + kCartBase,
// outside the spherical m range): field 7 holds the (l, nprim) sort order.
constexpr int kCartBase = 1000;
__device__ __forceinline__ void cart_powers(int l, int j, int& nx, int& ny, int& nz) {
  nx = l;
  while (nx > 0 && j >= l - nx + 1) {
    j -= l - nx + 1;
    --nx;
  }
  ny = l - nx - j;
  nz = j;
}

// P = x^nx y^ny z^nz, its gradient G and Laplacian (not zero: P is not harmonic)
template <class R>
__device__ __forceinline__ R cart_mono(R x, R y, R z, int nx, int ny, int nz) {
  return jq_pow(x, nx) * jq_pow(y, ny) * jq_pow(z, nz);
}

template <class R>
__device__ __forceinline__ void cart_mono_gl(R x, R y, R z, int nx, int ny, int nz, R& P, R* G, R& lap) {
  const R px = jq_pow(x, nx), py = jq_pow(y, ny), pz = jq_pow(z, nz);
  const R d1x = nx > 0 ? R(nx) * jq_pow(x, nx - 1) : R(0), d1y = ny > 0 ? R(ny) * jq_pow(y, ny - 1) : R(0);
  const R d1z = nz > 0 ? R(nz) * jq_pow(z, nz - 1) : R(0);
  const R d2x = nx > 1 ? R(nx * (nx - 1)) * jq_pow(x, nx - 2) : R(0), d2y = ny > 1 ? R(ny * (ny - 1)) * jq_pow(y, ny - 2) : R(0);
  const R d2z = nz > 1 ? R(nz * (nz - 1)) * jq_pow(z, nz - 2) : R(0);
  P = px * py * pz;
  G[0] = d1x * py * pz;
  G[1] = px * d1y * pz;
  G[2] = px * py * d1z;
  lap = d2x * py * pz + px * d2y * pz + px * py * d2z;
}

// d = p - R_atom in double (no cancellation), then rounded to R
template <class R>
__device__ __forceinline__ void disp(const double* apos, int atom, double px, double py, double pz, R& dx, R& dy, R& dz) {
  dx = (R)(px - apos[3 * atom]);
  dy = (R)(py - apos[3 * atom + 1]);
  dz = (R)(pz - apos[3 * atom + 2]);
}

template <class R, class F>
__device__ __forceinline__ void shell_val_d(const Basis& b, int s, R dx, R dy, R dz, F& f) {
  const int* sh = b.shells + kSh * s;
  const int l = sh[1], np = sh[2], p0 = sh[3], ao0 = sh[4], nm = sh[5], jlo = sh[6] + sh[1];
  const R r2 = dx * dx + dy * dy + dz * dz;
  const R* pr = prims_of<R>(b) + 2 * p0;
  R rad = R(0);
  for (int p = 0; p < np; ++p) rad += pr[2 * p + 1] * Num<R>::ex(-pr[2 * p] * r2);
  if (sh[6] >= kCartBase) {
    int nx, ny, nz;
    cart_powers(l, sh[6] - kCartBase, nx, ny, nz);
    f(ao0, rad * cart_mono(dx, dy, dz, nx, ny, nz));
    return;
  }
  switch (l) {
    case 0: emit_val<0, R>(dx, dy, dz, rad, ao0, jlo, nm, f); break;
    case 1: emit_val<1, R>(dx, dy, dz, rad, ao0, jlo, nm, f); break;
    case 2: emit_val<2, R>(dx, dy, dz, rad, ao0, jlo, nm, f); break;
    case 3: emit_val<3, R>(dx, dy, dz, rad, ao0, jlo, nm, f); break;
    case 4: emit_val<4, R>(dx, dy, dz, rad, ao0, jlo, nm, f); break;
    case 5: emit_val<5, R>(dx, dy, dz, rad, ao0, jlo, nm, f); break;
    default: emit_val<6, R>(dx, dy, dz, rad, ao0, jlo, nm, f); break;
  }
}

template <class R, class F>
__device__ __forceinline__ void shell_vgl_d(const Basis& b, int s, R dx, R dy, R dz, F& f) {
  const int* sh = b.shells + kSh * s;
  const int l = sh[1], np = sh[2], p0 = sh[3], ao0 = sh[4], nm = sh[5], jlo = sh[6] + sh[1];
  const R r2 = dx * dx + dy * dy + dz * dz;
  const R* pr = prims_of<R>(b) + 2 * p0;
  R rad = R(0), radZ = R(0), radZ2 = R(0);
  for (int p = 0; p < np; ++p) {
    const R Z = pr[2 * p];
    const R e = pr[2 * p + 1] * Num<R>::ex(-Z * r2);
    rad += e;
    radZ += Z * e;
    radZ2 += Z * Z * e;
  }
  if (sh[6] >= kCartBase) {   // grad = rad grad P - 2 radZ P d; lap = P (4 r^2 radZ2 - (4l+6) radZ) + rad lap P (d . grad P = l P)
    int nx, ny, nz;
    cart_powers(l, sh[6] - kCartBase, nx, ny, nz);
    R P, G[3], lp;
    cart_mono_gl(dx, dy, dz, nx, ny, nz, P, G, lp);
    const R t = R(-2) * radZ * P;
    f(ao0, rad * P, rad * G[0] + t * dx, rad * G[1] + t * dy, rad * G[2] + t * dz,
      P * (R(4) * r2 * radZ2 - (R(4 * l) + R(6)) * radZ) + rad * lp);
    return;
  }
  switch (l) {
    case 0: emit_vgl<0, R>(dx, dy, dz, r2, rad, radZ, radZ2, ao0, jlo, nm, f); break;
    case 1: emit_vgl<1, R>(dx, dy, dz, r2, rad, radZ, radZ2, ao0, jlo, nm, f); break;
    case 2: emit_vgl<2, R>(dx, dy, dz, r2, rad, radZ, radZ2, ao0, jlo, nm, f); break;
    case 3: emit_vgl<3, R>(dx, dy, dz, r2, rad, radZ, radZ2, ao0, jlo, nm, f); break;
    case 4: emit_vgl<4, R>(dx, dy, dz, r2, rad, radZ, radZ2, ao0, jlo, nm, f); break;
    case 5: emit_vgl<5, R>(dx, dy, dz, r2, rad, radZ, radZ2, ao0, jlo, nm, f); break;
    default: emit_vgl<6, R>(dx, dy, dz, r2, rad, radZ, radZ2, ao0, jlo, nm, f); break;
  }
}

// P points at once: sum_{a in shell} phi_a(d_p) v[a] into acc[p].  The points
// share the shell's primitive table and the v entries (loaded once); the P
// evaluations are independent, which gives each lane P chains of work.
// LO: the table also has low parts vlo (v + vlo is the FP64-accurate value);
// their products are added as a correction.
template <int L, int P, class R, class V, class Acc, bool LO = false>
__device__ __forceinline__ void emit_dot_pts(const R* dx, const R* dy, const R* dz, const R* rad, int ao0, int jlo, int nm,
                                             const V* v, Acc* acc, const float* vlo = nullptr) {
  R vv[2 * L + 1];
  R vl[LO ? 2 * L + 1 : 1];
#pragma unroll
  for (int j = 0; j < 2 * L + 1; ++j) {
    const int k = j - jlo;
    vv[j] = (k >= 0 && k < nm) ? (R)v[ao0 + k] : R(0);
    if constexpr (LO) vl[j] = (k >= 0 && k < nm) ? (R)vlo[ao0 + k] : R(0);
  }
#pragma unroll
  for (int p = 0; p < P; ++p) {
    R S[2 * L + 1];
    sh_val<L, R>(dx[p], dy[p], dz[p], S);
    R part = R(0);
#pragma unroll
    for (int j = 0; j < 2 * L + 1; ++j) part += S[j] * vv[j];
    acc_fma(acc[p], rad[p], part);
    if constexpr (LO) {
      R plo = R(0);
#pragma unroll
      for (int j = 0; j < 2 * L + 1; ++j) plo += S[j] * vl[j];
      acc_add(acc[p], rad[p] * plo);
    }
    if constexpr (AccTraits<Acc>::accurate) {
      R pabs = R(0);
#pragma unroll
      for (int j = 0; j < 2 * L + 1; ++j) pabs += fabs(S[j] * vv[j]);
      acc_mag(acc[p], fabs(rad[p]) * pabs);
    }
  }
}

template <int P, class R, class V, class Acc, bool LO = false>
__device__ __forceinline__ void shell_dot_pts(const Basis& b, int s, const R* dx, const R* dy, const R* dz, const V* v, Acc* acc,
                                              const float* vlo = nullptr) {
  const int* sh = b.shells + kSh * s;
  const int l = sh[1], np = sh[2], p0 = sh[3], ao0 = sh[4], nm = sh[5], jlo = sh[6] + sh[1];
  const R* pr = prims_of<R>(b) + 2 * p0;
  R r2[P], rad[P];
#pragma unroll
  for (int p = 0; p < P; ++p) {
    r2[p] = dx[p] * dx[p] + dy[p] * dy[p] + dz[p] * dz[p];
    rad[p] = R(0);
  }
  for (int q = 0; q < np; ++q) {
    const R Z = pr[2 * q], c = pr[2 * q + 1];
#pragma unroll
    for (int p = 0; p < P; ++p) rad[p] += c * MeshExp<R, AccTraits<Acc>::accurate>::ex(-Z * r2[p]);
  }
  if (sh[6] >= kCartBase) {
    int nx, ny, nz;
    cart_powers(l, sh[6] - kCartBase, nx, ny, nz);
    const R vv = (R)v[ao0];
#pragma unroll
    for (int p = 0; p < P; ++p) {
      const R t = cart_mono(dx[p], dy[p], dz[p], nx, ny, nz) * vv;
      acc_fma(acc[p], rad[p], t);
      if constexpr (AccTraits<Acc>::accurate) acc_mag(acc[p], fabs(rad[p]) * fabs(t));
    }
    return;
  }
  switch (l) {
    case 0: emit_dot_pts<0, P, R, V, Acc, LO>(dx, dy, dz, rad, ao0, jlo, nm, v, acc, vlo); break;
    case 1: emit_dot_pts<1, P, R, V, Acc, LO>(dx, dy, dz, rad, ao0, jlo, nm, v, acc, vlo); break;
    case 2: emit_dot_pts<2, P, R, V, Acc, LO>(dx, dy, dz, rad, ao0, jlo, nm, v, acc, vlo); break;
    case 3: emit_dot_pts<3, P, R, V, Acc, LO>(dx, dy, dz, rad, ao0, jlo, nm, v, acc, vlo); break;
    case 4: emit_dot_pts<4, P, R, V, Acc, LO>(dx, dy, dz, rad, ao0, jlo, nm, v, acc, vlo); break;
    case 5: emit_dot_pts<5, P, R, V, Acc, LO>(dx, dy, dz, rad, ao0, jlo, nm, v, acc, vlo); break;
    default: emit_dot_pts<6, P, R, V, Acc, LO>(dx, dy, dz, rad, ao0, jlo, nm, v, acc, vlo); break;
  }
}

// shell_dot_pts with the squared distances given as float-float pairs
// (r2h + r2l): exp(-Z (r2h + r2l)) = expf(-Z r2h) (1 - Z r2l) to second order,
// so that the float AO values carry only the rounding of their own evaluation.
template <int P, class V, class Acc, bool LO = false>
__device__ __forceinline__ void shell_dot_pts_ff(const Basis& b, int s, const float* dx, const float* dy, const float* dz,
                                                 const float* r2h, const float* r2l, const V* v, Acc* acc,
                                                 const float* vlo = nullptr) {
  const int* sh = b.shells + kSh * s;
  const int l = sh[1], np = sh[2], p0 = sh[3], ao0 = sh[4], nm = sh[5], jlo = sh[6] + sh[1];
  const float* pr = b.primsf + 2 * p0;
  float rad[P];
#pragma unroll
  for (int p = 0; p < P; ++p) rad[p] = 0.f;
  for (int q = 0; q < np; ++q) {
    const float Z = pr[2 * q], c = pr[2 * q + 1];
#pragma unroll
    for (int p = 0; p < P; ++p) rad[p] += c * expf(-Z * r2h[p]) * (1.f - Z * r2l[p]);
  }
  if (sh[6] >= kCartBase) {
    int nx, ny, nz;
    cart_powers(l, sh[6] - kCartBase, nx, ny, nz);
    const float vv = (float)v[ao0];
#pragma unroll
    for (int p = 0; p < P; ++p) {
      const float t = cart_mono(dx[p], dy[p], dz[p], nx, ny, nz) * vv;
      acc_fma(acc[p], rad[p], t);
      if constexpr (AccTraits<Acc>::accurate) acc_mag(acc[p], fabs(rad[p]) * fabs(t));
    }
    return;
  }
  switch (l) {
    case 0: emit_dot_pts<0, P, float, V, Acc, LO>(dx, dy, dz, rad, ao0, jlo, nm, v, acc, vlo); break;
    case 1: emit_dot_pts<1, P, float, V, Acc, LO>(dx, dy, dz, rad, ao0, jlo, nm, v, acc, vlo); break;
    case 2: emit_dot_pts<2, P, float, V, Acc, LO>(dx, dy, dz, rad, ao0, jlo, nm, v, acc, vlo); break;
    case 3: emit_dot_pts<3, P, float, V, Acc, LO>(dx, dy, dz, rad, ao0, jlo, nm, v, acc, vlo); break;
    case 4: emit_dot_pts<4, P, float, V, Acc, LO>(dx, dy, dz, rad, ao0, jlo, nm, v, acc, vlo); break;
    case 5: emit_dot_pts<5, P, float, V, Acc, LO>(dx, dy, dz, rad, ao0, jlo, nm, v, acc, vlo); break;
    default: emit_dot_pts<6, P, float, V, Acc, LO>(dx, dy, dz, rad, ao0, jlo, nm, v, acc, vlo); break;
  }
}

// d = (x0h + x0l) + m as a float pair (dh, dl) by TwoSum
__device__ __forceinline__ void ff_add(float x0h, float x0l, float m, float& dh, float& dl) {
  const float t = __fadd_rn(x0h, m);
  const float z = __fsub_rn(t, x0h);
  const float e = __fadd_rn(__fsub_rn(x0h, __fsub_rn(t, z)), __fsub_rn(m, z));
  dh = t;
  dl = e + x0l;
}

// |d|^2 for d = dh + dl (per component) as a float pair: exact squares of the
// high parts by FMA, the cross terms 2 dh dl, and the rounding of the sum
__device__ __forceinline__ void ff_r2(float xh, float xl, float yh, float yl, float zh, float zl, float& r2h, float& r2l) {
  const float px = __fmul_rn(xh, xh), py = __fmul_rn(yh, yh), pz = __fmul_rn(zh, zh);
  const float ex = __fmaf_rn(xh, xh, -px), ey = __fmaf_rn(yh, yh, -py), ez = __fmaf_rn(zh, zh, -pz);
  const float s1 = __fadd_rn(px, py);
  const float z1 = __fsub_rn(s1, px);
  const float e1 = __fadd_rn(__fsub_rn(px, __fsub_rn(s1, z1)), __fsub_rn(py, z1));
  const float s2 = __fadd_rn(s1, pz);
  const float z2 = __fsub_rn(s2, s1);
  const float e2 = __fadd_rn(__fsub_rn(s1, __fsub_rn(s2, z2)), __fsub_rn(pz, z2));
  r2h = s2;
  r2l = (ex + ey + ez) + (e1 + e2) + 2.f * (xh * xl + yh * yl + zh * zl);
}

// Visit every AO of a basis at point p (shells are grouped by nucleus, so the
// displacement is recomputed only when the nucleus changes).
template <class R, class F>
__device__ __forceinline__ void ao_visit(const Basis& b, const double* apos, double px, double py, double pz, F& f) {
  int last = -1;
  R dx = R(0), dy = R(0), dz = R(0);
  for (int s = 0; s < b.nshell; ++s) {
    const int atom = b.shells[kSh * s];
    if (atom != last) {
      disp<R>(apos, atom, px, py, pz, dx, dy, dz);
      last = atom;
    }
    shell_val_d<R>(b, s, dx, dy, dz, f);
  }
}

template <class R, class F>
__device__ __forceinline__ void ao_visit_vgl(const Basis& b, const double* apos, double px, double py, double pz, F& f) {
  int last = -1;
  R dx = R(0), dy = R(0), dz = R(0);
  for (int s = 0; s < b.nshell; ++s) {
    const int atom = b.shells[kSh * s];
    if (atom != last) {
      disp<R>(apos, atom, px, py, pz, dx, dy, dz);
      last = atom;
    }
    shell_vgl_d<R>(b, s, dx, dy, dz, f);
  }
}

// all AO values at one point into out[] (block-cooperative, split by shell; no
// sync).  Shells whose reach (e^-40) ends short of the point write zeros.
template <class R, class V>
__device__ void ao_fill_block(const Basis& b, const double* apos, double px, double py, double pz, V* out) {
  auto f = [&](int a, R val) { out[a] = (V)val; };
  for (int s = threadIdx.x; s < b.nshell; s += blockDim.x) {
    R dx, dy, dz;
    disp<R>(apos, b.shells[kSh * s], px, py, pz, dx, dy, dz);
    if ((float)(dx * dx + dy * dy + dz * dz) > __int_as_float(b.shells[kSh * s + kShReach])) {
      for (int a = 0; a < b.shells[kSh * s + 5]; ++a) out[b.shells[kSh * s + 4] + a] = (V)0;
      continue;
    }
    shell_val_d<R>(b, s, dx, dy, dz, f);
  }
}

// ------------------------------------------------------------------ reductions

// Sum over the block; every thread receives the total.  red: >= 33 doubles.
__device__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < nw; ++k) t += red[k];
    red[32] = t;
  }
  __syncthreads();
  return red[32];
}

__device__ double block_min(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = red[0];
    for (int k = 1; k < nw; ++k) t = fmin(t, red[k]);
    red[32] = t;
  }
  __syncthreads();
  return red[32];
}

// out[k] = sum_a M[k*A + a] x[a] for k < n (one warp per row)
template <class T>
__device__ void rows_dot(const T* __restrict__ M, int n, int A, const T* __restrict__ x, T* out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = wid; k < n; k += nw) {
    const T* row = M + (size_t)k * A;
    T acc0 = T(0), acc1 = T(0);
    int a = lane;
    for (; a + 32 < A; a += 64) {   // two independent loads in flight per lane
      acc0 += row[a] * x[a];
      acc1 += row[a + 32] * x[a + 32];
    }
    if (a < A) acc0 += row[a] * x[a];
    const T acc = warp_sum(acc0 + acc1);
    if (lane == 0) out[k] = acc;
  }
}

// Loads kept in flight per thread by the column helpers below.
constexpr int kMLP = 4;

// v[j*A + b] += c[j] * x for j < n (one column b of a table): the loads of a
// group of kMLP rows are issued before their stores, so a thread keeps kMLP
// memory requests in flight instead of one load-modify-store at a time.
template <class Tab>
__device__ __forceinline__ void column_axpy(Tab* __restrict__ v, size_t A, int b, int n, const Tab* __restrict__ c, Tab x) {
  for (int j0 = 0; j0 < n; j0 += kMLP) {
    Tab t[kMLP];
#pragma unroll
    for (int u = 0; u < kMLP; ++u)
      if (j0 + u < n) t[u] = v[(size_t)(j0 + u) * A + b];
#pragma unroll
    for (int u = 0; u < kMLP; ++u)
      if (j0 + u < n) v[(size_t)(j0 + u) * A + b] = t[u] + c[j0 + u] * x;
  }
}

// sum_j v[j*A + b] c[j] with kMLP partial sums
template <class Tab>
__device__ __forceinline__ Tab column_dot(const Tab* __restrict__ v, size_t A, int b, int n, const Tab* __restrict__ c) {
  Tab acc[kMLP];
#pragma unroll
  for (int u = 0; u < kMLP; ++u) acc[u] = Tab(0);
  for (int j0 = 0; j0 < n; j0 += kMLP) {
#pragma unroll
    for (int u = 0; u < kMLP; ++u)
      if (j0 + u < n) acc[u] += v[(size_t)(j0 + u) * A + b] * c[j0 + u];
  }
  Tab r = Tab(0);
#pragma unroll
  for (int u = 0; u < kMLP; ++u) r += acc[u];
  return r;
}

// sum_a L[a*A + b] x[a] (column b of a row-major A x A matrix) with kMLP partial sums
template <class Tab>
__device__ __forceinline__ Tab matvec_col(const Tab* __restrict__ L, int A, int b, const Tab* __restrict__ x) {
  Tab acc[kMLP];
#pragma unroll
  for (int u = 0; u < kMLP; ++u) acc[u] = Tab(0);
  int a = 0;
  for (; a + kMLP <= A; a += kMLP) {
#pragma unroll
    for (int u = 0; u < kMLP; ++u) acc[u] += L[(size_t)(a + u) * A + b] * x[a + u];
  }
  for (; a < A; ++a) acc[0] += L[(size_t)a * A + b] * x[a];
  Tab r = Tab(0);
#pragma unroll
  for (int u = 0; u < kMLP; ++u) r += acc[u];
  return r;
}

// ------------------------------------------------------------------ physics helpers
template <class R>
__device__ __forceinline__ R j2_pair(int type, R b, R d) {
  if (type == 0) return d / R(2) * (R(1) / (R(1) + b * d));
  return R(1) / (R(2) * b) * (R(1) - Num<R>::ex(-b * d));
}

// J1 at one point: sum over nuclei
template <class R>
__device__ R j1_at(const Sys& s, double x, double y, double z) {
  R acc = R(0);
  const R a = (R)s.j1_param;
  for (int at = 0; at < s.natom; ++at) {
    R dx, dy, dz;
    disp<R>(s.atom_pos, at, x, y, z, dx, dy, dz);
    const R d = Num<R>::sq(dx * dx + dy * dy + dz * dz);
    const R c = (R)s.j1_cA[2 * at], A = (R)s.j1_cA[2 * at + 1];
    if (s.j1_type == 0) acc += -A * (R(1) / (R(2) * a)) * (R(1) - Num<R>::ex(-a * c * d));
    else acc += -A * d / (R(2) * (R(1) + a * c * d));
  }
  return acc;
}

// sum over electrons m != skip of the J2 pair function at distance |p - r_m|
template <class R>
__device__ R j2_at(const Sys& s, const double* r, int skip, double x, double y, double z) {
  R acc = R(0);
  const R b = (R)s.j2_param;
  for (int m = 0; m < s.N; ++m) {
    if (m == skip) continue;
    const R dx = (R)(x - r[3 * m]), dy = (R)(y - r[3 * m + 1]), dz = (R)(z - r[3 * m + 2]);
    acc += j2_pair<R>(s.j2_type, b, Num<R>::sq(dx * dx + dy * dy + dz * dz));
  }
  return acc;
}

__device__ __forceinline__ double ipow(double x, double n) {
  const int k = (int)n;
  if ((double)k == n && k >= 0 && k <= 8) {
    double r = 1.0;
    for (int i = 0; i < k; ++i) r *= x;
    return r;
  }
  return pow(x, n);
}

// r^-2 sum_k c_k r^{n_k} exp(-alpha_k r^2) over the terms of (atom, slot)
__device__ double ecp_channel(const Sys& s, int atom, int slot, double d) {
  const int* ch = s.ecp_chan + (atom * kSlots + slot) * 2;
  double v = 0.0;
  for (int t = 0; t < ch[1]; ++t) {
    const double* tm = s.ecp_terms + 3 * (ch[0] + t);
    v += tm[0] * ipow(d, tm[1]) * exp(-tm[2] * d * d);
  }
  return v / (d * d);
}

template <class T>
__device__ __forceinline__ T legendre_t(int l, T x) {
  switch (l) {
    case 0: return T(1);
    case 1: return x;
    case 2: return T(0.5) * (T(3) * x * x - T(1));
    case 3: return T(0.5) * (T(5) * x * x * x - T(3) * x);
    case 4: return T(0.125) * (T(35) * x * x * x * x - T(30) * x * x + T(3));
    case 5: return T(0.125) * (T(63) * x * x * x * x * x - T(70) * x * x * x + T(15) * x);
    default: return T(0.0625) * (T(231) * x * x * x * x * x * x - T(315) * x * x * x * x + T(105) * x * x - T(5));
  }
}

// nearest nucleus (lowest index on ties), as the stable argsort of jqmc/structure.py:393-405
__device__ int nearest_atom(const Sys& s, double x, double y, double z) {
  int best = 0;
  double bd = 1e300;
  for (int a = 0; a < s.natom; ++a) {
    const double dx = s.atom_pos[3 * a] - x, dy = s.atom_pos[3 * a + 1] - y, dz = s.atom_pos[3 * a + 2] - z;
    const double d = sqrt(dx * dx + dy * dy + dz * dz);
    if (d < bd) { bd = d; best = a; }
  }
  return best;
}

// R(alpha, beta, gamma) of jqmc_mcmc.py:4228-4245 / jqmc_gfmc.py:4721-4736
__device__ void rotation(double a, double b, double g, double* R) {
  const double ca = cos(a), sa = sin(a), cb = cos(b), sb = sin(b), cg = cos(g), sg = sin(g);
  R[0] = cb * cg; R[1] = cg * sa * sb - ca * sg; R[2] = sa * sg + ca * cg * sb;
  R[3] = cb * sg; R[4] = ca * cg + sa * sb * sg; R[5] = ca * sb * sg - cg * sa;
  R[6] = -sb;     R[7] = cb * sa;                R[8] = ca * cb;
}

// Derivative tables of one electron at (x, y, z), computed in double and stored
// in Tab: dp[c*A + a] = (grad x, y, z, lap)_c of geminal AO a; dp3[c*A3 + a] =
// (value, grad x, y, z, lap)_c of J3 AO a.  Block-cooperative over shells, no sync.
// Shells whose reach (e^-40 for the values) ends short of the point write zeros.
template <class Tab>
__device__ void fill_dtables(const Sys& s, double x, double y, double z, Tab* dp, Tab* dp3) {
  const int A = s.det.nao;
  for (int sh = threadIdx.x; sh < s.det.nshell; sh += blockDim.x) {
    double dx, dy, dz;
    disp<double>(s.atom_pos, s.det.shells[kSh * sh], x, y, z, dx, dy, dz);
    auto f = [&](int a, double v, double gx, double gy, double gz, double lp) {
      dp[a] = (Tab)gx; dp[A + a] = (Tab)gy; dp[2 * A + a] = (Tab)gz; dp[3 * A + a] = (Tab)lp;
    };
    if ((float)(dx * dx + dy * dy + dz * dz) > __int_as_float(s.det.shells[kSh * sh + kShReach])) {
      for (int a = 0; a < s.det.shells[kSh * sh + 5]; ++a) f(s.det.shells[kSh * sh + 4] + a, 0.0, 0.0, 0.0, 0.0, 0.0);
      continue;
    }
    shell_vgl_d<double>(s.det, sh, dx, dy, dz, f);
  }
  if (s.has_j3) {
    const int A3 = s.j3.nao;
    for (int sh = threadIdx.x; sh < s.j3.nshell; sh += blockDim.x) {
      double dx, dy, dz;
      disp<double>(s.atom_pos, s.j3.shells[kSh * sh], x, y, z, dx, dy, dz);
      auto f = [&](int a, double v, double gx, double gy, double gz, double lp) {
        dp3[a] = (Tab)v; dp3[A3 + a] = (Tab)gx; dp3[2 * A3 + a] = (Tab)gy; dp3[3 * A3 + a] = (Tab)gz; dp3[4 * A3 + a] = (Tab)lp;
      };
      if ((float)(dx * dx + dy * dy + dz * dz) > __int_as_float(s.j3.shells[kSh * sh + kShReach])) {
        for (int a = 0; a < s.j3.shells[kSh * sh + 5]; ++a) f(s.j3.shells[kSh * sh + 4] + a, 0.0, 0.0, 0.0, 0.0, 0.0);
        continue;
      }
      shell_vgl_d<double>(s.j3, sh, dx, dy, dz, f);
    }
  }
}

// J2 pair function derivatives f'(d), f''(d)
__device__ __forceinline__ void j2_pair_d(const Sys& s, double d, double& f1, double& f2) {
  const double b = s.j2_param;
  if (s.j2_type == 0) {
    const double q = 1.0 + b * d;
    f1 = 1.0 / (2.0 * q * q);
    f2 = -b / (q * q * q);
  } else {
    const double ex = exp(-b * d);
    f1 = 0.5 * ex;
    f2 = -0.5 * b * ex;
  }
}

// The one-electron fields of an energy-cache row at (x, y, z): e-ion Coulomb
// (coulomb_potential.py:2285-2328), local ECP (coulomb_potential.py:1145-1246),
// grad/lap J1 (jastrow_factor.py:961-1034), nearest nucleus and the non-local
// channel values there (coulomb_potential.py:1478-1712 with NN = 1).
__device__ void ecache_single(const Sys& s, double x, double y, double z, double* row) {
  double ei = 0.0, eloc = 0.0, gx = 0.0, gy = 0.0, gz = 0.0, lap = 0.0, bd = 1e300;
  int best = 0;
  for (int a = 0; a < s.natom; ++a) {
    const double dx = x - s.atom_pos[3 * a], dy = y - s.atom_pos[3 * a + 1], dz = z - s.atom_pos[3 * a + 2];
    const double d = sqrt(dx * dx + dy * dy + dz * dz);
    if (d < bd) { bd = d; best = a; }
    ei += -s.atom_zeff[a] / d;
    if (s.ecp_flag) eloc += ecp_channel(s, a, s.ecp_maxl1[a], d);
    if (s.has_j1) {
      const double aa = s.j1_param, c = s.j1_cA[2 * a], AA = s.j1_cA[2 * a + 1];
      double f1, f2;
      if (s.j1_type == 0) {
        const double ex = exp(-aa * c * d);
        f1 = -AA * c * ex / 2.0;
        f2 = AA * aa * c * c * ex / 2.0;
      } else {
        const double q = 1.0 + aa * c * d;
        f1 = -AA / (2.0 * q * q);
        f2 = AA * aa * c / (q * q * q);
      }
      gx += f1 * dx / d; gy += f1 * dy / d; gz += f1 * dz / d;
      lap += f2 + 2.0 * f1 / d;
    }
  }
  row[EC_EI] = ei;
  row[EC_ELOC] = eloc;
  row[EC_J1G] = gx; row[EC_J1G + 1] = gy; row[EC_J1G + 2] = gz;
  row[EC_J1L] = lap;
  row[EC_NEAR] = (double)best;
  row[EC_DIST] = bd;
  const int lmax = s.ecp_flag ? s.ecp_maxl1[best] : 0;
  for (int l = 0; l < kSlots; ++l) row[EC_VL + l] = l < lmax ? ecp_channel(s, best, l, bd) : 0.0;
}

// The same row computed by one warp (every lane calls it): lanes over nuclei,
// warp sums, the nearest nucleus as the (distance, index) minimum (lowest index
// on ties, as the serial loop), and the channel values at it by lanes over l.
__device__ void ecache_single_warp(const Sys& s, double x, double y, double z, double* row) {
  const int lane = threadIdx.x & 31;
  double ei = 0.0, eloc = 0.0, gx = 0.0, gy = 0.0, gz = 0.0, lap = 0.0, bd = 1e300;
  int best = 0x7fffffff;
  for (int a = lane; a < s.natom; a += 32) {
    const double dx = x - s.atom_pos[3 * a], dy = y - s.atom_pos[3 * a + 1], dz = z - s.atom_pos[3 * a + 2];
    const double d = sqrt(dx * dx + dy * dy + dz * dz);
    if (d < bd) { bd = d; best = a; }
    ei += -s.atom_zeff[a] / d;
    if (s.ecp_flag) eloc += ecp_channel(s, a, s.ecp_maxl1[a], d);
    if (s.has_j1) {
      const double aa = s.j1_param, c = s.j1_cA[2 * a], AA = s.j1_cA[2 * a + 1];
      double f1, f2;
      if (s.j1_type == 0) {
        const double ex = exp(-aa * c * d);
        f1 = -AA * c * ex / 2.0;
        f2 = AA * aa * c * c * ex / 2.0;
      } else {
        const double q = 1.0 + aa * c * d;
        f1 = -AA / (2.0 * q * q);
        f2 = AA * aa * c / (q * q * q);
      }
      gx += f1 * dx / d; gy += f1 * dy / d; gz += f1 * dz / d;
      lap += f2 + 2.0 * f1 / d;
    }
  }
  ei = warp_sum(ei); eloc = warp_sum(eloc);
  gx = warp_sum(gx); gy = warp_sum(gy); gz = warp_sum(gz); lap = warp_sum(lap);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double od = __shfl_xor_sync(0xffffffffu, bd, o);
    const int ob = __shfl_xor_sync(0xffffffffu, best, o);
    if (od < bd || (od == bd && ob < best)) { bd = od; best = ob; }
  }
  if (lane == 0) {
    row[EC_EI] = ei;
    row[EC_ELOC] = eloc;
    row[EC_J1G] = gx; row[EC_J1G + 1] = gy; row[EC_J1G + 2] = gz;
    row[EC_J1L] = lap;
    row[EC_NEAR] = (double)best;
    row[EC_DIST] = bd;
  }
  const int lmax = s.ecp_flag ? s.ecp_maxl1[best] : 0;
  if (lane < kSlots) row[EC_VL + lane] = lane < lmax ? ecp_channel(s, best, lane, bd) : 0.0;
}

// Fill the whole energy cache of one walker from its positions (block-cooperative).
__device__ void ecache_init(const Sys& s, const double* r, double* ec, double* red) {
  const int N = s.N;
  for (int e = threadIdx.x; e < N; e += blockDim.x) {
    double* row = ec + (size_t)e * kEC;
    ecache_single(s, r[3 * e], r[3 * e + 1], r[3 * e + 2], row);
    double gx = 0.0, gy = 0.0, gz = 0.0, lap = 0.0;
    if (s.has_j2)
      for (int m = 0; m < N; ++m) {
        if (m == e) continue;
        const double dx = r[3 * e] - r[3 * m], dy = r[3 * e + 1] - r[3 * m + 1], dz = r[3 * e + 2] - r[3 * m + 2];
        const double d = sqrt(dx * dx + dy * dy + dz * dz);
        double f1, f2;
        j2_pair_d(s, d, f1, f2);
        gx += f1 * dx / d; gy += f1 * dy / d; gz += f1 * dz / d;
        lap += f2 + 2.0 * f1 / d;
      }
    row[EC_J2G] = gx; row[EC_J2G + 1] = gy; row[EC_J2G + 2] = gz;
    row[EC_J2L] = lap;
  }
  double ee = 0.0;
  for (int p = threadIdx.x; p < N * N; p += blockDim.x) {
    const int a = p / N, b = p % N;
    if (b <= a) continue;
    const double dx = r[3 * a] - r[3 * b], dy = r[3 * a + 1] - r[3 * b + 1], dz = r[3 * a + 2] - r[3 * b + 2];
    ee += 1.0 / sqrt(dx * dx + dy * dy + dz * dz);
  }
  ee = block_sum(ee, red);
  if (threadIdx.x == 0) ec[(size_t)N * kEC + EC_TOT_EE] = ee;
}

// ------------------------------------------------------------------ per-walker workspace
template <class Tab>
struct Work {
  Sys s;
  int N, n, A, A3;
  double* r;     // N*3 (shared)
  Tab* G;        // n*n (shared)
  Tab* Gi;       // n*n (shared)
  Tab* Tup;      // global, this walker
  Tab* Tdn;
  Tab* h3;
  Tab* dphi;     // global: N x 4 x A  (grad x, y, z, lap of the geminal AOs at each electron)
  Tab* dphi3;    // global: N x 5 x A3 (value, grad x, y, z, lap of the J3 AOs at each electron)
  double* ec;    // global: (N + 1) x kEC energy cache
  Tab* vA0;      // A (shared)
  Tab* vA1;
  Tab* vA2;
  Tab* v30;      // A3 (shared)
  Tab* v31;
  Tab* v32;
  Tab* vn0;      // n (shared)
  Tab* vn1;
  Tab* vn2;
  Tab* vn3;
  double* red;   // kRed
  double* sc;    // 32 scalars
  const float* tlo_up;   // mixed form: low parts of T_up / T_dn and of the J3 field
  const float* tlo_dn;   // from the last build (nullptr when the tables have moved
  const float* h3lo;     // since, or are not kept); h3lo is nullptr without J3
};

struct WorkLayout {
  int off_r, off_G, off_Gi, off_vA, off_v3, off_vn, off_red, off_sc, bytes;
};

// Shared-memory offsets of the walker (re)initialisation (after the staged tables)
struct InitLayout {
  int r, red, sc, Gd, aug, vec, bytes;
};

WorkLayout work_layout(const Sys& s, int base, int tab_bytes) {
  WorkLayout L;
  const int A3 = s.has_j3 ? s.j3.nao : 1;
  int o = base;
  L.off_r = o; o = align16(o + s.N * 3 * 8);
  L.off_G = o; o = align16(o + s.n_up * s.n_up * tab_bytes);
  L.off_Gi = o; o = align16(o + s.n_up * s.n_up * tab_bytes);
  L.off_vA = o; o = align16(o + 3 * s.det.nao * tab_bytes);
  L.off_v3 = o; o = align16(o + 3 * A3 * tab_bytes);
  L.off_vn = o; o = align16(o + 4 * s.n_up * tab_bytes);
  L.off_red = o; o = align16(o + kRed * 8);
  L.off_sc = o; o = align16(o + 32 * 8);
  L.bytes = o;
  return L;
}

template <class Tab>
__device__ Work<Tab> make_work(const Sys& s, const WorkLayout& L, unsigned char* smem, const WS& ws, int w) {
  Work<Tab> k;
  k.s = s;
  k.N = s.N;
  k.n = s.n_up;
  k.A = s.det.nao;
  k.A3 = s.has_j3 ? s.j3.nao : 1;
  k.r = reinterpret_cast<double*>(smem + L.off_r);
  k.G = reinterpret_cast<Tab*>(smem + L.off_G);
  k.Gi = reinterpret_cast<Tab*>(smem + L.off_Gi);
  k.vA0 = reinterpret_cast<Tab*>(smem + L.off_vA);
  k.vA1 = k.vA0 + k.A;
  k.vA2 = k.vA1 + k.A;
  k.v30 = reinterpret_cast<Tab*>(smem + L.off_v3);
  k.v31 = k.v30 + k.A3;
  k.v32 = k.v31 + k.A3;
  k.vn0 = reinterpret_cast<Tab*>(smem + L.off_vn);
  k.vn1 = k.vn0 + k.n;
  k.vn2 = k.vn1 + k.n;
  k.vn3 = k.vn2 + k.n;
  k.red = reinterpret_cast<double*>(smem + L.off_red);
  k.sc = reinterpret_cast<double*>(smem + L.off_sc);
  k.Tup = static_cast<Tab*>(ws.Tup) + (size_t)w * k.n * k.A;
  k.Tdn = static_cast<Tab*>(ws.Tdn) + (size_t)w * k.n * k.A;
  k.h3 = s.has_j3 ? static_cast<Tab*>(ws.h3) + (size_t)w * k.N * k.A3 : nullptr;
  k.dphi = static_cast<Tab*>(ws.dphi) + (size_t)w * k.N * 4 * k.A;
  k.dphi3 = s.has_j3 ? static_cast<Tab*>(ws.dphi3) + (size_t)w * k.N * 5 * k.A3 : nullptr;
  k.ec = ws.ecache + (size_t)w * (k.N + 1) * kEC;
  k.tlo_up = ws.tlo ? ws.tlo + (size_t)w * tlo_stride(s) : nullptr;
  k.tlo_dn = ws.tlo ? k.tlo_up + (size_t)k.n * k.A : nullptr;
  k.h3lo = ws.tlo && s.has_j3 ? k.tlo_up + (size_t)2 * k.n * k.A : nullptr;
  return k;
}

template <class Tab>
__device__ void load_walker(Work<Tab>& k, const WS& ws, int w) {
  const int nn = k.n * k.n;
  for (int t = threadIdx.x; t < k.N * 3; t += blockDim.x) k.r[t] = ws.r[(size_t)w * k.N * 3 + t];
  const Tab* G = static_cast<const Tab*>(ws.G) + (size_t)w * nn;
  const Tab* Gi = static_cast<const Tab*>(ws.Ginv) + (size_t)w * nn;
  for (int t = threadIdx.x; t < nn; t += blockDim.x) {
    k.G[t] = G[t];
    k.Gi[t] = Gi[t];
  }
  __syncthreads();
}

template <class Tab>
__device__ void store_walker(const Work<Tab>& k, const WS& ws, int w) {
  __syncthreads();
  const int nn = k.n * k.n;
  Tab* G = static_cast<Tab*>(ws.G) + (size_t)w * nn;
  Tab* Gi = static_cast<Tab*>(ws.Ginv) + (size_t)w * nn;
  for (int t = threadIdx.x; t < k.N * 3; t += blockDim.x) ws.r[(size_t)w * k.N * 3 + t] = k.r[t];
  for (int t = threadIdx.x; t < nn; t += blockDim.x) {
    G[t] = k.G[t];
    Gi[t] = k.Gi[t];
  }
}

// Move electron e (global index, up first) to (px, py, pz) and patch G, G^-1,
// T_up, T_dn and the J3 field.  Block-cooperative; returns the det ratio.
//   up i:  a = T_up phi',  ratio = a_i,  w = a - e_i,  g' = a^T G (new row i),
//          G^-1 -= G^-1[:,i] w^T / ratio,  T_up -= T_up[i] (x) w / ratio,
//          T_dn += G^-1[:,i] (x) (lambda^T dphi - T_dn^T G^T w) / ratio
//   dn j:  b = T_dn phi', ratio = b_j,  q = b - e_j,  c' = G b (new column j),
//          G^-1 -= q G^-1[j,:] / ratio, T_dn -= q (x) T_dn[j] / ratio,
//          T_up += G^-1[j,:] (x) (lambda dphi - T_up^T G q) / ratio
// (every right-hand side uses the tables before the move).  Arithmetic in Tab.
template <class Tab, bool CACHES = true>
__device__ double sm_move(Work<Tab>& k, int e, double px, double py, double pz) {
  const Sys& s = k.s;
  const int n = k.n, A = k.A, A3 = k.A3;
  const bool up = e < s.n_up;
  const int i = up ? e : e - s.n_up;
  const double ox = k.r[3 * e], oy = k.r[3 * e + 1], oz = k.r[3 * e + 2];
  const Tab* lam = lam_of<Tab>(s);
  const Tab* lamT = lamT_of<Tab>(s);
  // phi' -> vA0, phi_old -> vA1, then vA1 = dphi
  ao_fill_block<Tab, Tab>(s.det, s.atom_pos, px, py, pz, k.vA0);
  ao_fill_block<Tab, Tab>(s.det, s.atom_pos, ox, oy, oz, k.vA1);
  if (s.has_j3) {
    ao_fill_block<Tab, Tab>(s.j3, s.atom_pos, px, py, pz, k.v30);
    ao_fill_block<Tab, Tab>(s.j3, s.atom_pos, ox, oy, oz, k.v31);
  }
  __syncthreads();
  for (int a = threadIdx.x; a < A; a += blockDim.x) k.vA1[a] = k.vA0[a] - k.vA1[a];
  if (s.has_j3)
    for (int a = threadIdx.x; a < A3; a += blockDim.x) k.v31[a] = k.v30[a] - k.v31[a];
  rows_dot<Tab>(up ? k.Tup : k.Tdn, n, A, k.vA0, k.vn0);
  __syncthreads();
  const Tab ratio = k.vn0[i];
  const Tab inv = Tab(1) / ratio;
  Tab* scn = reinterpret_cast<Tab*>(k.sc);  // 32 doubles of scratch
  const int scn_cap = (int)(32 * sizeof(double) / sizeof(Tab));
  if (up) {
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      k.vn1[t] = k.vn0[t] - (t == i ? Tab(1) : Tab(0));
      k.vn3[t] = k.Gi[t * n + i];
    }
    __syncthreads();
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      Tab u = Tab(0);
      for (int t = 0; t < n; ++t) u += k.G[t * n + c] * k.vn1[t];
      k.vn2[c] = u;
    }
    __syncthreads();
    for (int b = threadIdx.x; b < A; b += blockDim.x) {
      const Tab dl = matvec_col<Tab>(lam, A, b, k.vA1);
      const Tab mw = column_dot<Tab>(k.Tdn, A, b, n, k.vn2);
      k.vA2[b] = (dl - mw) * inv;
    }
    __syncthreads();
    for (int b = threadIdx.x; b < A; b += blockDim.x) {
      column_axpy<Tab>(k.Tdn, A, b, n, k.vn3, k.vA2[b]);
      const Tab ti = k.Tup[(size_t)i * A + b];
      column_axpy<Tab>(k.Tup, A, b, n, k.vn1, -ti * inv);
    }
    Tab* gn = (n <= scn_cap) ? scn : k.vA2;
    __syncthreads();
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      Tab g = Tab(0);
      for (int t = 0; t < n; ++t) g += k.vn0[t] * k.G[t * n + c];
      gn[c] = g;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      const int rr = t / n, cc = t % n;
      k.Gi[t] -= k.vn3[rr] * k.vn1[cc] * inv;
    }
    for (int c = threadIdx.x; c < n; c += blockDim.x) k.G[i * n + c] = gn[c];
  } else {
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      k.vn1[t] = k.vn0[t] - (t == i ? Tab(1) : Tab(0));
      k.vn3[t] = k.Gi[i * n + t];
    }
    __syncthreads();
    for (int rr = threadIdx.x; rr < n; rr += blockDim.x) {
      Tab u = Tab(0);
      for (int t = 0; t < n; ++t) u += k.G[rr * n + t] * k.vn1[t];
      k.vn2[rr] = u;
    }
    __syncthreads();
    for (int a = threadIdx.x; a < A; a += blockDim.x) {
      const Tab dm = matvec_col<Tab>(lamT, A, a, k.vA1);
      const Tab mq = column_dot<Tab>(k.Tup, A, a, n, k.vn2);
      k.vA2[a] = (dm - mq) * inv;
    }
    __syncthreads();
    for (int a = threadIdx.x; a < A; a += blockDim.x) {
      column_axpy<Tab>(k.Tup, A, a, n, k.vn3, k.vA2[a]);
      const Tab tj = k.Tdn[(size_t)i * A + a];
      column_axpy<Tab>(k.Tdn, A, a, n, k.vn1, -tj * inv);
    }
    Tab* cn = (n <= scn_cap) ? scn : k.vA2;
    __syncthreads();
    for (int rr = threadIdx.x; rr < n; rr += blockDim.x) {
      Tab c = Tab(0);
      for (int t = 0; t < n; ++t) c += k.G[rr * n + t] * k.vn0[t];
      cn[rr] = c;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      const int rr = t / n, cc = t % n;
      k.Gi[t] -= k.vn1[rr] * k.vn3[cc] * inv;
    }
    for (int rr = threadIdx.x; rr < n; rr += blockDim.x) k.G[rr * n + i] = cn[rr];
  }
  // J3 field: h_m += J dphi3 or J^T dphi3 for every other electron m
  if (s.has_j3) {
    const Tab* J = j3m_of<Tab>(s);
    const Tab* JT = j3mT_of<Tab>(s);
    __syncthreads();
    for (int c = threadIdx.x; c < A3; c += blockDim.x) {
      Tab jd = Tab(0), jtd = Tab(0);
      for (int cp = 0; cp < A3; ++cp) {
        jd += JT[(size_t)cp * A3 + c] * k.v31[cp];   // (J d)_c
        jtd += J[(size_t)cp * A3 + c] * k.v31[cp];   // (J^T d)_c
      }
      k.v32[c] = jd;
      k.v30[c] = jtd;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < k.N * A3; t += blockDim.x) {
      const int m = t / A3, c = t % A3;
      if (m == e) continue;
      const bool mup = m < s.n_up;
      bool useJ;  // h_m += J d  iff the pair is (phi_m^T J phi_e)
      if (mup == up) useJ = m < e;
      else useJ = !up;  // e dn, m up -> phi_m^T J phi_e
      k.h3[(size_t)m * A3 + c] += useJ ? k.v32[c] : k.v30[c];
    }
  }
  if constexpr (CACHES) {
    fill_dtables<Tab>(s, px, py, pz, k.dphi + (size_t)e * 4 * A, s.has_j3 ? k.dphi3 + (size_t)e * 5 * A3 : nullptr);
    // energy cache: every pair with the moved electron (J2 terms of the partner,
    // e-e Coulomb), then the moved electron's own row
    {
      const int N = k.N;
      double dee = 0.0, jgx = 0.0, jgy = 0.0, jgz = 0.0, jl = 0.0;
      for (int m = threadIdx.x; m < N; m += blockDim.x) {
        if (m == e) continue;
        const double mx = k.r[3 * m], my = k.r[3 * m + 1], mz = k.r[3 * m + 2];
        const double oxm = mx - ox, oym = my - oy, ozm = mz - oz;      // r_m - r_e(old)
        const double nxm = mx - px, nym = my - py, nzm = mz - pz;      // r_m - r_e(new)
        const double dold = sqrt(oxm * oxm + oym * oym + ozm * ozm);
        const double dnew = sqrt(nxm * nxm + nym * nym + nzm * nzm);
        dee += 1.0 / dnew - 1.0 / dold;
        if (s.has_j2) {
          double f1o, f2o, f1n, f2n;
          j2_pair_d(s, dold, f1o, f2o);
          j2_pair_d(s, dnew, f1n, f2n);
          double* row = k.ec + (size_t)m * kEC;
          row[EC_J2G] += f1n * nxm / dnew - f1o * oxm / dold;
          row[EC_J2G + 1] += f1n * nym / dnew - f1o * oym / dold;
          row[EC_J2G + 2] += f1n * nzm / dnew - f1o * ozm / dold;
          row[EC_J2L] += (f2n + 2.0 * f1n / dnew) - (f2o + 2.0 * f1o / dold);
          jgx -= f1n * nxm / dnew; jgy -= f1n * nym / dnew; jgz -= f1n * nzm / dnew;
          jl += f2n + 2.0 * f1n / dnew;
        }
      }
      dee = block_sum(dee, k.red);
      jgx = block_sum(jgx, k.red);
      jgy = block_sum(jgy, k.red);
      jgz = block_sum(jgz, k.red);
      jl = block_sum(jl, k.red);
      if (threadIdx.x < 32) {
        double* row = k.ec + (size_t)e * kEC;
        ecache_single_warp(s, px, py, pz, row);
        if (threadIdx.x == 0) {
          row[EC_J2G] = jgx; row[EC_J2G + 1] = jgy; row[EC_J2G + 2] = jgz;
          row[EC_J2L] = jl;
          k.ec[(size_t)N * kEC + EC_TOT_EE] += dee;
        }
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    k.r[3 * e] = px;
    k.r[3 * e + 1] = py;
    k.r[3 * e + 2] = pz;
  }
  __syncthreads();
  return (double)ratio;
}

// ------------------------------------------------------------------ per-step terms
// Arrays in shared memory for the energy / projection kernels.
struct Terms {
  double* ke;     // N continuum kinetic energy per electron
  double* c3;     // N  phi3(r_e) . h_e
  double* ei;     // N  e-ion Coulomb per electron
  double* eid;    // N  discretised e-ion (distance floor alat)
  double* edist;  // N  distance to the nearest nucleus
  int* eatom;     // N  nearest nucleus
  double* el;     // 6N kinetic lattice elements
  double* V;      // nv*N non-local ECP elements
  float* vm;      // N  compensated energy: sum over the electron's ECP points of |w_v| M_v
  uint16_t* act;  // kMaxWarps x (det + J3 shells): each warp's list of shells within reach
  double* R;      // 9 rotation
  float* Rf;      // mixed form: 9 rotation + nv x (g_x, g_y, g_z, 1/|g|) rotated quadrature directions, float
  float* dA;      // mixed form: N*natom*3  float(r_e - R_a)
  float* dE;      // mixed form: N*N*3      float(r_e - r_m)
};

// Warps per CTA of the walker kernels with FP64 mesh ratios (the only ones that
// keep shell lists: the FP64 kernels and the block energy's FP64 refinement);
// the float projection launches without the list slots.
constexpr int kMaxWarps = 8;
static_assert(LrdmcShape<double, double>::threads / 32 <= kMaxWarps && LrdmcShape<float, F2>::threads / 32 <= kMaxWarps,
              "shell-list slots for every warp");

struct TermsLayout {
  int off_ke, off_c3, off_ei, off_eid, off_ed, off_ea, off_el, off_V, off_vm, off_R, off_Rf, off_dA, off_dE, off_act,
      act_warp, bytes;
};

// rel: reserve the float displacement caches of the mixed form in shared memory
TermsLayout terms_layout(const Sys& s, int base, bool rel) {
  TermsLayout L;
  const int N = s.N;
  int o = base;
  L.off_ke = o; o = align16(o + N * 8);
  L.off_c3 = o; o = align16(o + N * 8);
  L.off_ei = o; o = align16(o + N * 8);
  L.off_eid = o; o = align16(o + N * 8);
  L.off_ed = o; o = align16(o + N * 8);
  L.off_ea = o; o = align16(o + N * 4);
  L.off_el = o; o = align16(o + 6 * N * 8);
  L.off_V = o; o = align16(o + (s.nv > 0 ? s.nv : 1) * N * 8);
  L.off_vm = o; o = align16(o + N * 4);
  L.off_R = o; o = align16(o + 9 * 8);
  L.off_Rf = o; o = align16(o + (9 + 4 * (s.nv > 0 ? s.nv : 1)) * 4);
  L.off_dA = o; o = align16(o + (rel ? N * s.natom * 3 * 4 : 0));
  L.off_dE = o; o = align16(o + (rel ? N * N * 3 * 4 : 0));
  // last, so that a kernel of fewer warps launches with less of it
  L.act_warp = align16((s.det.nshell + (s.has_j3 ? s.j3.nshell : 0)) * 2);
  L.off_act = o; o += kMaxWarps * L.act_warp;
  L.bytes = o;
  return L;
}

// Dynamic shared memory of a walker kernel whose FP64 mesh ratios run in
// `threads` threads per CTA (0: no FP64 mesh ratios, no shell lists).
int terms_smem(const TermsLayout& L, int threads) { return L.bytes - (kMaxWarps - threads / 32) * L.act_warp; }

// Displacement caches bigger than this live in global memory (per walker).
constexpr int kDcacheSmemMax = 64 * 1024;

bool is_mixed(int precision) { return precision == JQMC_PREC_MIXED || precision == JQMC_PREC_MIXED_FASTE; }

int dcache_bytes(const Sys& s) { return s.N * (s.natom + s.N) * 3 * 4; }

__device__ Terms make_terms(const TermsLayout& L, unsigned char* smem, float* gdcache, const Sys& s) {
  Terms t;
  t.ke = reinterpret_cast<double*>(smem + L.off_ke);
  t.c3 = reinterpret_cast<double*>(smem + L.off_c3);
  t.ei = reinterpret_cast<double*>(smem + L.off_ei);
  t.eid = reinterpret_cast<double*>(smem + L.off_eid);
  t.edist = reinterpret_cast<double*>(smem + L.off_ed);
  t.eatom = reinterpret_cast<int*>(smem + L.off_ea);
  t.el = reinterpret_cast<double*>(smem + L.off_el);
  t.V = reinterpret_cast<double*>(smem + L.off_V);
  t.vm = reinterpret_cast<float*>(smem + L.off_vm);
  t.act = reinterpret_cast<uint16_t*>(smem + L.off_act);
  t.R = reinterpret_cast<double*>(smem + L.off_R);
  t.Rf = reinterpret_cast<float*>(smem + L.off_Rf);
  t.dA = L.off_dE > L.off_dA ? reinterpret_cast<float*>(smem + L.off_dA) : nullptr;
  t.dE = L.bytes > L.off_dE ? reinterpret_cast<float*>(smem + L.off_dE) : nullptr;
  if (gdcache) {
    t.dA = gdcache;
    t.dE = gdcache + (size_t)s.N * s.natom * 3;
  }
  return t;
}

// Float displacement caches of the mixed form: dA[e][a] = r_e - R_a,
// dE[e][m] = r_e - r_m (differences in double, rounded once).  Filled at the
// start of a launch, then only the moved electron's row and column change.
template <class Tab>
__device__ void dcache_fill(const Work<Tab>& k, Terms& t) {
  if (!t.dA) return;
  const Sys& s = k.s;
  const int M = s.natom, N = k.N;
  for (int p = threadIdx.x; p < N * (M + N); p += blockDim.x) {
    const int e = p / (M + N), q = p % (M + N);
    const double* X = q < M ? s.atom_pos + 3 * q : k.r + 3 * (q - M);
    float* out = q < M ? t.dA + (size_t)(e * M + q) * 3 : t.dE + (size_t)(e * N + q - M) * 3;
    out[0] = (float)(k.r[3 * e] - X[0]);
    out[1] = (float)(k.r[3 * e + 1] - X[1]);
    out[2] = (float)(k.r[3 * e + 2] - X[2]);
  }
  __syncthreads();
}

template <class Tab>
__device__ void dcache_update(const Work<Tab>& k, Terms& t, int e) {
  if (!t.dA) return;
  const Sys& s = k.s;
  const int M = s.natom, N = k.N;
  const double ex = k.r[3 * e], ey = k.r[3 * e + 1], ez = k.r[3 * e + 2];
  for (int q = threadIdx.x; q < M + 2 * N; q += blockDim.x) {
    float* out;
    double dx, dy, dz;
    if (q < M) {
      out = t.dA + (size_t)(e * M + q) * 3;
      dx = ex - s.atom_pos[3 * q]; dy = ey - s.atom_pos[3 * q + 1]; dz = ez - s.atom_pos[3 * q + 2];
    } else if (q < M + N) {
      const int m = q - M;
      out = t.dE + (size_t)(e * N + m) * 3;
      dx = ex - k.r[3 * m]; dy = ey - k.r[3 * m + 1]; dz = ez - k.r[3 * m + 2];
    } else {
      const int m = q - M - N;
      out = t.dE + (size_t)(m * N + e) * 3;
      dx = k.r[3 * m] - ex; dy = k.r[3 * m + 1] - ey; dz = k.r[3 * m + 2] - ez;
    }
    out[0] = (float)dx; out[1] = (float)dy; out[2] = (float)dz;
  }
  __syncthreads();
}

// The determinant part of electron e's derivatives at FP64 accuracy, for the
// The shells (positions in the (l, nprim)-sorted order) whose reach radius
// extends to within `margin` of electron e: every mesh point p of the electron
// with |p - r_e| <= margin is then beyond the reach of every other shell, whose
// AOs are below e^-kReach there and are left out of the ratio.  One warp; the
// list goes to the warp's slot of t.act.
struct ShellList {
  const uint16_t* det;
  int ndet;
  const uint16_t* j3;
  int nj3;
};

template <class Tab>
__device__ ShellList shell_list(const Work<Tab>& k, const Terms& t, int e, float margin) {
  const Sys& s = k.s;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint16_t* buf = t.act + (size_t)wid * (s.det.nshell + (s.has_j3 ? s.j3.nshell : 0));
  auto build = [&](const Basis& b, uint16_t* out) -> int {
    int cnt = 0;
    for (int base = 0; base < b.nshell; base += 32) {
      const int idx = base + lane;
      bool keep = false;
      if (idx < b.nshell) {
        const int sh = b.shells[kSh * idx + 7];
        const int atom = b.shells[kSh * sh];
        const double x = k.r[3 * e] - s.atom_pos[3 * atom], y = k.r[3 * e + 1] - s.atom_pos[3 * atom + 1];
        const double z = k.r[3 * e + 2] - s.atom_pos[3 * atom + 2];
        const float dd = fmaxf(sqrtf((float)(x * x + y * y + z * z)) - margin, 0.f);
        keep = dd * dd < __int_as_float(b.shells[kSh * sh + kShReach]);
      }
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (keep) out[cnt + __popc(m & ((1u << lane) - 1u))] = (uint16_t)idx;
      cnt += __popc(m);
    }
    return cnt;
  };
  __syncwarp();   // the previous list is no longer read
  ShellList L;
  L.det = buf;
  L.ndet = build(s.det, buf);
  L.j3 = buf + s.det.nshell;
  L.nj3 = s.has_j3 ? build(s.j3, buf + s.det.nshell) : 0;
  __syncwarp();
  return L;
}

// block energy of the mixed form right after a build: the AO values, gradients
// and Laplacians of basis b re-evaluated in FP64 at r_e (the float tables hold
// them rounded, which alone moves E_L by about 1e-5 Ha on the 30-electron ring)
// dotted with the FP64-accurate row v_hi + v_lo (a T row, or a J3 field row).
// One warp; the lanes split the shells; every lane returns (value, grad x, y, z,
// Laplacian) of phi . v.
template <class Tab>
__device__ void dot_vgl_fp64(const Sys& s, const Basis& b, const double* re, const Tab* v, const float* vlo, double* out) {
  const int lane = threadIdx.x & 31;
  double a0 = 0.0, ax = 0.0, ay = 0.0, az = 0.0, al = 0.0;
  auto f = [&](int a, double val, double gx, double gy, double gz, double lap) {
    const double t = (double)v[a] + (double)vlo[a];
    a0 += val * t; ax += gx * t; ay += gy * t; az += gz * t; al += lap * t;
  };
  for (int idx = lane; idx < b.nshell; idx += 32) {
    const int sh = b.shells[kSh * idx + 7];
    double dx, dy, dz;
    disp<double>(s.atom_pos, b.shells[kSh * sh], re[0], re[1], re[2], dx, dy, dz);
    shell_vgl_d<double>(b, sh, dx, dy, dz, f);
  }
  out[0] = warp_sum(a0); out[1] = warp_sum(ax); out[2] = warp_sum(ay); out[3] = warp_sum(az); out[4] = warp_sum(al);
}

// Phase A: per-electron continuum kinetic energy and the old-position values
// the ratios need (wavefunction.py:1142-1207 with jastrow_factor.py:961-1034,
// 3435-3558, 4077-4156).  One warp per electron: the cached AO derivative tables
// are dotted with the electron's T row and J3 field (lane and warp sums in the
// accumulation type Acc); J1/J2 derivatives, Coulomb and ECP terms come
// from the energy cache.
template <class Tab, class Acc = Tab>
__device__ void electron_terms(Work<Tab>& k, Terms& t, double alat) {
  using Out = typename AccTraits<Acc>::out;
  using Ar = typename AccTraits<Acc>::arith;
  const Sys& s = k.s;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int A = k.A, A3 = k.A3;
  // Each warp walks its electrons; lane (it mod 32) keeps the it-th electron's
  // nine sums, and every 32 electrons (and at the end) all holding lanes finish
  // their electron's terms in double at once, so the FP64 work issues once per
  // 32 electrons instead of once per electron.
  Out kp[9];
  int mine = -1, it = 0;
  for (int e = wid; e < k.N; e += nw, ++it) {
    const bool up = e < s.n_up;
    const int i = up ? e : e - s.n_up;
    const Tab* Trow = (up ? k.Tup : k.Tdn) + (size_t)i * A;
    const Tab* dp = k.dphi + (size_t)e * 4 * A;
    if (e + nw < k.N) {   // this warp's next electron: its derivative tables and T row
      const int en = e + nw;
      prefetch_l2(k.dphi + (size_t)en * 4 * A, (size_t)4 * A * sizeof(Tab), lane);
      prefetch_l2((en < s.n_up ? k.Tup + (size_t)en * A : k.Tdn + (size_t)(en - s.n_up) * A), (size_t)A * sizeof(Tab), lane);
      if (s.has_j3) prefetch_l2(k.dphi3 + (size_t)en * 5 * A3, (size_t)5 * A3 * sizeof(Tab), lane);
    }
    Acc tgx, tgy, tgz, tlp, tc3, thx, thy, thz, thl;
    acc_zero(tgx); acc_zero(tgy); acc_zero(tgz); acc_zero(tlp);
    acc_zero(tc3); acc_zero(thx); acc_zero(thy); acc_zero(thz); acc_zero(thl);
    // the block energy of the mixed form on fresh tables: FP64-accurate
    // determinant terms (the float projection keeps the table dots)
    constexpr bool kMayRefine = sizeof(Tab) == sizeof(float) && !std::is_same<Acc, float>::value;
    const float* Tlo = kMayRefine ? (up ? k.tlo_up : k.tlo_dn) : nullptr;
    double dt[5] = {0.0, 0.0, 0.0, 0.0, 0.0}, d3[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (kMayRefine && Tlo) {
      dot_vgl_fp64(s, s.det, k.r + 3 * e, Trow, Tlo + (size_t)i * A, dt);
    } else {
      for (int a = lane; a < A; a += 32) {
        const Ar tv = (Ar)Trow[a];
        acc_fma(tgx, (Ar)dp[a], tv);
        acc_fma(tgy, (Ar)dp[A + a], tv);
        acc_fma(tgz, (Ar)dp[2 * A + a], tv);
        acc_fma(tlp, (Ar)dp[3 * A + a], tv);
      }
    }
    if (kMayRefine && Tlo && k.h3lo) {
      dot_vgl_fp64(s, s.j3, k.r + 3 * e, k.h3 + (size_t)e * A3, k.h3lo + (size_t)e * A3, d3);
    } else if (s.has_j3) {
      const Tab* h = k.h3 + (size_t)e * A3;
      const Tab* q = k.dphi3 + (size_t)e * 5 * A3;
      for (int a = lane; a < A3; a += 32) {
        const Ar hv = (Ar)h[a];
        acc_fma(tc3, (Ar)q[a], hv);
        acc_fma(thx, (Ar)q[A3 + a], hv);
        acc_fma(thy, (Ar)q[2 * A3 + a], hv);
        acc_fma(thz, (Ar)q[3 * A3 + a], hv);
        acc_fma(thl, (Ar)q[4 * A3 + a], hv);
      }
    }
    Out v0 = acc_out(tgx), v1 = acc_out(tgy), v2 = acc_out(tgz), v3 = acc_out(tlp);
    if (kMayRefine && Tlo) { v0 = (Out)dt[1]; v1 = (Out)dt[2]; v2 = (Out)dt[3]; v3 = (Out)dt[4]; }
    Out v4 = acc_out(tc3), v5 = acc_out(thx), v6 = acc_out(thy), v7 = acc_out(thz), v8 = acc_out(thl);
    if (kMayRefine && Tlo && k.h3lo) { v4 = (Out)d3[0]; v5 = (Out)d3[1]; v6 = (Out)d3[2]; v7 = (Out)d3[3]; v8 = (Out)d3[4]; }
    if (lane == (it & 31)) {
      kp[0] = v0; kp[1] = v1; kp[2] = v2; kp[3] = v3; kp[4] = v4; kp[5] = v5; kp[6] = v6; kp[7] = v7; kp[8] = v8;
      mine = e;
    }
    if ((it & 31) == 31 || e + nw >= k.N) {
      if (mine >= 0) {
        const int me = mine;
        const double gx = (double)kp[0], gy = (double)kp[1], gz = (double)kp[2], lp = (double)kp[3];
        const double c3 = (double)kp[4], hx = (double)kp[5], hy = (double)kp[6], hz = (double)kp[7], hl = (double)kp[8];
        const double* row = k.ec + (size_t)me * kEC;
        const double Gx = gx + hx + row[EC_J1G] + row[EC_J2G];
        const double Gy = gy + hy + row[EC_J1G + 1] + row[EC_J2G + 1];
        const double Gz = gz + hz + row[EC_J1G + 2] + row[EC_J2G + 2];
        const double L = lp - (gx * gx + gy * gy + gz * gz) + hl + row[EC_J1L] + row[EC_J2L];
        t.ke[me] = -0.5 * (L + Gx * Gx + Gy * Gy + Gz * Gz);
        t.c3[me] = c3;
        t.ei[me] = row[EC_EI];
        t.eatom[me] = (int)row[EC_NEAR];
        t.edist[me] = row[EC_DIST];
        if (s.ecp_flag && s.ecp_maxl1[(int)row[EC_NEAR]] <= 0)
          for (int v = 0; v < s.nv; ++v) t.V[me * s.nv + v] = 0.0;
        if (!s.ecp_flag) {
          const double x = k.r[3 * me], y = k.r[3 * me + 1], z = k.r[3 * me + 2];
          double eid = 0.0;
          for (int a = 0; a < s.natom; ++a) {
            const double dx = x - s.atom_pos[3 * a], dy = y - s.atom_pos[3 * a + 1], dz = z - s.atom_pos[3 * a + 2];
            eid += -s.atom_zeff[a] / fmax(sqrt(dx * dx + dy * dy + dz * dz), alat);
          }
          t.eid[me] = eid;
        }
      }
      mine = -1;
    }
  }
  __syncthreads();
}

// One J1 / J2 pair term of J(r_e + s) - J(r_e): d0 = r_e - X, move s; the
// difference is formed from r'^2 - r^2 = (2 d0 + s).s so that small moves keep
// their relative accuracy (jastrow_factor.py:649-726, 1181-1251).
template <class R, bool ACC = false>
__device__ __forceinline__ R pair_delta(R d0x, R d0y, R d0z, R sx, R sy, R sz, int type, R a, R c, R A, bool j1) {
  using E = MeshExp<R, ACC>;
  const R r2 = d0x * d0x + d0y * d0y + d0z * d0z;
  const R dr2 = (R(2) * d0x + sx) * sx + (R(2) * d0y + sy) * sy + (R(2) * d0z + sz) * sz;
  const R rr = Num<R>::sq(r2);
  const R rp2 = r2 + dr2;
  const R rp = Num<R>::sq(rp2 > R(0) ? rp2 : R(0));
  const R dr = (rp + rr > R(0)) ? dr2 / (rp + rr) : R(0);
  if (j1) {
    if (type == 0) return A / (R(2) * a) * E::ex(-a * c * rr) * E::em1(-a * c * dr);
    return -A * dr / (R(2) * (R(1) + a * c * rr) * (R(1) + a * c * rp));
  }
  if (type == 0) return dr / (R(2) * (R(1) + a * rr) * (R(1) + a * rp));
  return -E::ex(-a * rr) * E::em1(-a * dr) / (R(2) * a);
}

// psi(r_e + s_p)/psi(r) for P moves s_p of electron e (det x Jastrow),
// arithmetic in R, one warp: the lanes split the geminal and J3 shells, the
// nuclei (J1) and the other electrons (J2); every lane returns all P ratios.
// In the mixed form (R = float) the electron displacements come from the float
// caches t.dA / t.dE; otherwise from the positions in double.
template <int P, class R, class Tab, class Acc>
__device__ void wf_ratio_pts(const Work<Tab>& k, const Terms& t, int e, const R* sx, const R* sy, const R* sz,
                             typename AccTraits<Acc>::out* ratio, float* mag = nullptr, const float* sl = nullptr,
                             bool dlt = false, unsigned vneg = 0u, const ShellList* lst = nullptr) {
  using Out = typename AccTraits<Acc>::out;
  const Sys& s = k.s;
  const int lane = threadIdx.x & 31;
  const bool up = e < s.n_up;
  // the shells walked: those in the list, else all
  const int ndet = lst ? lst->ndet : s.det.nshell, nj3 = lst ? lst->nj3 : (s.has_j3 ? s.j3.nshell : 0);
  auto det_at = [&](int q) { return lst ? (int)lst->det[q] : q; };
  auto j3_at = [&](int q) { return lst ? (int)lst->j3[q] : q; };
  const int i = up ? e : e - s.n_up;
  const Tab* Trow = (up ? k.Tup : k.Tdn) + (size_t)i * k.A;
  // block energy on fresh tables (mixed form): the T row's low parts as well
  constexpr bool kMayRefine = sizeof(Tab) == sizeof(float) && !std::is_same<Acc, float>::value;
  const float* Tlo = nullptr;
  const float* hlo = nullptr;   // the J3 field row's low parts
  if constexpr (kMayRefine) {
    Tlo = (up ? k.tlo_up : k.tlo_dn) ? (up ? k.tlo_up : k.tlo_dn) + (size_t)i * k.A : nullptr;
    hlo = Tlo && k.h3lo ? k.h3lo + (size_t)e * k.A3 : nullptr;
  }
  const bool rel = sizeof(R) == sizeof(float) && t.dA != nullptr;
  const float* dAe = rel ? t.dA + (size_t)e * s.natom * 3 : nullptr;
  const float* dEe = rel ? t.dE + (size_t)e * k.N * 3 : nullptr;
  const double ex = k.r[3 * e], ey = k.r[3 * e + 1], ez = k.r[3 * e + 2];
  auto dnuc = [&](int atom, R& x, R& y, R& z) {
    if (rel) {
      x = (R)dAe[3 * atom]; y = (R)dAe[3 * atom + 1]; z = (R)dAe[3 * atom + 2];
    } else {
      x = (R)(ex - s.atom_pos[3 * atom]); y = (R)(ey - s.atom_pos[3 * atom + 1]); z = (R)(ez - s.atom_pos[3 * atom + 2]);
    }
  };
  const R* mx = sx;
  const R* my = sy;
  const R* mz = sz;
  Acc det[P], dj[P];
#pragma unroll
  for (int p = 0; p < P; ++p) { acc_zero(det[p]); acc_zero(dj[p]); }
  R dx[P], dy[P], dz[P];
  if constexpr (sizeof(R) == sizeof(float) && AccTraits<Acc>::accurate) {
    // compensated energy: displacements as float pairs (the low part from the
    // double positions), squared distances as float pairs
    float dxl[P], dyl[P], dzl[P], r2h[P], r2l[P];
    auto shells = [&](const Basis& b, const Tab* v, Acc* acc, const float* vlo, bool isj3) {
      const int nsh = isj3 ? nj3 : ndet;
      for (int q = lane; q < nsh; q += 32) {
        const int idx = isj3 ? j3_at(q) : det_at(q);
        const int sh = b.shells[kSh * idx + 7];
        const int atom = b.shells[kSh * sh];
        R x, y, z;
        dnuc(atom, x, y, z);
        const float xl = (float)((ex - s.atom_pos[3 * atom]) - (double)x);
        const float yl = (float)((ey - s.atom_pos[3 * atom + 1]) - (double)y);
        const float zl = (float)((ez - s.atom_pos[3 * atom + 2]) - (double)z);
#pragma unroll
        for (int p = 0; p < P; ++p) {
          ff_add(x, xl + sl[p], mx[p], dx[p], dxl[p]);
          ff_add(y, yl + sl[P + p], my[p], dy[p], dyl[p]);
          ff_add(z, zl + sl[2 * P + p], mz[p], dz[p], dzl[p]);
          ff_r2(dx[p], dxl[p], dy[p], dyl[p], dz[p], dzl[p], r2h[p], r2l[p]);
        }
        if (vlo) shell_dot_pts_ff<P, Tab, Acc, true>(b, sh, dx, dy, dz, r2h, r2l, v, acc, vlo);
        else shell_dot_pts_ff<P>(b, sh, dx, dy, dz, r2h, r2l, v, acc);
      }
    };
    shells(s.det, Trow, det, Tlo, false);
    if (s.has_j3) shells(s.j3, k.h3 + (size_t)e * k.A3, dj, hlo, true);
  } else {
    for (int q = lane; q < ndet; q += 32) {
      const int sh = s.det.shells[kSh * det_at(q) + 7];   // (l, nprim)-sorted order
      R x, y, z;
      dnuc(s.det.shells[kSh * sh], x, y, z);
#pragma unroll
      for (int p = 0; p < P; ++p) { dx[p] = x + mx[p]; dy[p] = y + my[p]; dz[p] = z + mz[p]; }
      if constexpr (kMayRefine) {
        if (Tlo) shell_dot_pts<P, R, Tab, Acc, true>(s.det, sh, dx, dy, dz, Trow, det, Tlo);
        else shell_dot_pts<P, R>(s.det, sh, dx, dy, dz, Trow, det);
      } else {
        shell_dot_pts<P, R>(s.det, sh, dx, dy, dz, Trow, det);
      }
    }
    if (s.has_j3) {
      const Tab* h = k.h3 + (size_t)e * k.A3;
      for (int q = lane; q < nj3; q += 32) {
        const int sh = s.j3.shells[kSh * j3_at(q) + 7];
        R x, y, z;
        dnuc(s.j3.shells[kSh * sh], x, y, z);
#pragma unroll
        for (int p = 0; p < P; ++p) { dx[p] = x + mx[p]; dy[p] = y + my[p]; dz[p] = z + mz[p]; }
        if constexpr (kMayRefine) {
          if (hlo) shell_dot_pts<P, R, Tab, Acc, true>(s.j3, sh, dx, dy, dz, h, dj, hlo);
          else shell_dot_pts<P, R>(s.j3, sh, dx, dy, dz, h, dj);
        } else {
          shell_dot_pts<P, R>(s.j3, sh, dx, dy, dz, h, dj);
        }
      }
    }
  }
  if (s.has_j1) {
    const R a = (R)s.j1_param;
    for (int at = lane; at < s.natom; at += 32) {
      R x, y, z;
      dnuc(at, x, y, z);
      const R c = (R)s.j1_cA[2 * at], A = (R)s.j1_cA[2 * at + 1];
#pragma unroll
      for (int p = 0; p < P; ++p) acc_add(dj[p], pair_delta<R, AccTraits<Acc>::accurate>(x, y, z, mx[p], my[p], mz[p], s.j1_type, a, c, A, true));
    }
  }
  if (s.has_j2) {
    const R b = (R)s.j2_param;
    for (int m = lane; m < k.N; m += 32) {
      if (m == e) continue;
      R x, y, z;
      if (rel) {
        x = (R)dEe[3 * m]; y = (R)dEe[3 * m + 1]; z = (R)dEe[3 * m + 2];
      } else {
        x = (R)(ex - k.r[3 * m]); y = (R)(ey - k.r[3 * m + 1]); z = (R)(ez - k.r[3 * m + 2]);
      }
#pragma unroll
      for (int p = 0; p < P; ++p) acc_add(dj[p], pair_delta<R, AccTraits<Acc>::accurate>(x, y, z, mx[p], my[p], mz[p], s.j2_type, b, R(0), R(0), false));
    }
  }
  const Out c3 = s.has_j3 ? (Out)t.c3[e] : Out(0);
#pragma unroll
  for (int p = 0; p < P; ++p) {
    const Out dsum = acc_out(det[p]);
    const Out jsum = acc_out(dj[p]);
    const Out jf = Num<Out>::ex(jsum - c3);
    ratio[p] = dsum * jf;
    if (dlt) {   // determinant locality: the Jastrow factor only where w_p det'/det < 0 (bit p of vneg: w_p < 0)
      const bool neg = ((vneg >> p) & 1u) ? (dsum > Out(0)) : (dsum < Out(0));
      if (!neg) ratio[p] = dsum;
    }
    if constexpr (AccTraits<Acc>::accurate) {
      if (mag) mag[p] = acc_mag_out(det[p]) * (float)jf;   // sum |phi_a T_a| on the ratio's scale
    }
  }
}

// Phase B: kinetic lattice elements (wavefunction.py:1740-1860) and non-local ECP
// elements (coulomb_potential.py:1478-1712, NN = 1).  Rotation R in t.R.  One
// warp per electron: its six lattice shifts, then its Nv quadrature points (if
// its nearest nucleus carries a non-local channel), P points per chunk (6 in
// float, 3 in double, for registers).
// The compensated block energy's error is dominated by walkers whose mesh
// ratios psi(r')/psi(r) = sum_a phi_a(r') T_a come out of large cancellations
// (near a node): the float rounding of the AO values is then relative to
// sum_a |phi_a T_a|, not to the ratio.  Per walker the element-weighted mean
// cancellation factor  C = sum_i |w_i| M_i / sum_i |w_i ratio_i|  (w_i the
// element's weight, M_i = sum_a |phi_a T_a| times its Jastrow factor) ranks the
// walkers by that error; its median is near 4 on sampled configurations.
struct Cancellation {
  float num = 0.f, den = 0.f;
  __device__ void add(float wabs, float mag, float el) {
    num += wabs * mag;
    den += fabsf(el);
  }
};

// Electrons whose ECP points have sum_v |w_v| M_v above this get their non-local
// elements again in FP64 in the block energy of the mixed form: with the float
// AO values off by a few 1e-8 relative, what the others leave is below about
// 3e-7 Ha per electron.
#ifndef JQMC_ECP_REFINE_MAG
#define JQMC_ECP_REFINE_MAG 32.0
#endif
constexpr double kEcpRefineMag = JQMC_ECP_REFINE_MAG;

// Returns this thread's shares of the walker's cancellation factor (compensated
// mode; zero otherwise).  The compensated mode also leaves per electron in t.vm
// the sum over its ECP points of |w_v| M_v (w_v the element's weight, M_v as in
// the cancellation factor): the float AO values' rounding moves the electron's
// non-local energy by a few 1e-8 of it.  With `refine` set, only the ECP points
// of the electrons with refine[e] > kEcpRefineMag are computed (again).
template <class R, class Tab, class Acc = R>
__device__ Cancellation mesh_terms(const Work<Tab>& k, Terms& t, double alat, bool kinetic, const float* refine = nullptr) {
  using Out = typename AccTraits<Acc>::out;
  constexpr bool kErr = AccTraits<Acc>::accurate;
  Cancellation cancel;
  constexpr int P = sizeof(R) == sizeof(float) ? 6 : 3;
  constexpr int nkc = 6 / P;   // chunks of lattice shifts
  const Sys& s = k.s;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int N = k.N, nv = s.nv;
  const double kin = -1.0 / (2.0 * alat * alat);
  for (int e = wid; e < N; e += nw) {
    if (refine && !(refine[e] > (float)kEcpRefineMag)) continue;   // (warp-uniform)
    const int atom = t.eatom[e];
    const bool ecp = s.ecp_flag && s.ecp_maxl1[atom] > 0;
    const int nchunk = nkc + (ecp ? (nv + P - 1) / P : 0);
    float vmag = 0.f;
    const bool lattice = kinetic && !refine;
    // FP64 ratios walk only the shells within reach of the electron's mesh
    // points, which lie within alat (lattice) and 2 |r_e - R_I| (quadrature
    // sphere around its nearest nucleus I) of r_e.  The float ratios walk every
    // shell: there the list costs more than the AO work it saves (measured on
    // the chain: 582 ms with lists against 486 ms without for 40 projections of
    // 4096 walkers; the FP64 projection gains 18 %).
    ShellList lst{nullptr, 0, nullptr, 0};
    if constexpr (sizeof(R) == sizeof(double)) {
      const float margin = fmaxf(lattice ? (float)alat : 0.f, ecp ? 2.f * (float)t.edist[e] : 0.f) + 1e-3f;
      lst = shell_list(k, t, e, margin);
    }
    const ShellList* lstp = sizeof(R) == sizeof(double) ? &lst : nullptr;
    if (e + nw < N) {   // this warp's next electron: its T row, J3 field and displacements
      const int en = e + nw;
      const Tab* Tn = (en < s.n_up ? k.Tup + (size_t)en * k.A : k.Tdn + (size_t)(en - s.n_up) * k.A);
      prefetch_l2(Tn, (size_t)k.A * sizeof(Tab), lane);
      if (s.has_j3) prefetch_l2(k.h3 + (size_t)en * k.A3, (size_t)k.A3 * sizeof(Tab), lane);
      if (sizeof(R) == sizeof(float) && t.dA && __isGlobal(t.dA)) {   // (a shared-memory cache needs none)
        prefetch_l2(t.dA + (size_t)en * s.natom * 3, (size_t)s.natom * 12, lane);
        prefetch_l2(t.dE + (size_t)en * N * 3, (size_t)N * 12, lane);
      }
    }
    for (int c = lattice ? 0 : nkc; c < nchunk; ++c) {
      // lane p < P sets up point p, then every lane receives all P moves.  The
      // float form builds them from the float rotation, quadrature directions
      // and displacement cache, so that the chunk issues no FP64 instruction.
      R mx = R(0), my = R(0), mz = R(0), ct = R(0);
      float mxl = 0.f, myl = 0.f, mzl = 0.f;   // compensated form: low parts of the move
      int v0 = 0, np = P;
      if (c >= nkc) {
        v0 = (c - nkc) * P;
        np = min(P, nv - v0);
      }
      if (lane < P) {
        if constexpr (sizeof(R) == sizeof(float) && !kErr) {
          if (c < nkc) {
            const int kk = c * P + lane, ax = kk >> 1;
            const float sg = (kk & 1) ? -(float)alat : (float)alat;
            mx = sg * t.Rf[ax]; my = sg * t.Rf[3 + ax]; mz = sg * t.Rf[6 + ax];
          } else {
            // rel = R - r; r' = r + rel + |rel| g ; cos = (-rel/|rel|) . (g/|g|)
            const float* dAe = t.dA + ((size_t)e * s.natom + atom) * 3;
            const float relx = -dAe[0], rely = -dAe[1], relz = -dAe[2];
            const float dist = sqrtf(relx * relx + rely * rely + relz * relz);
            const float* g = t.Rf + 9 + 4 * (lane < np ? v0 + lane : v0);
            ct = -(relx * g[0] + rely * g[1] + relz * g[2]) / dist * g[3];
            mx = relx + dist * g[0]; my = rely + dist * g[1]; mz = relz + dist * g[2];
          }
        } else {
          double dmx, dmy, dmz;
          if (c < nkc) {
            const int kk = c * P + lane, ax = kk >> 1;
            const double sg = (kk & 1) ? -alat : alat;
            dmx = sg * t.R[ax]; dmy = sg * t.R[3 + ax]; dmz = sg * t.R[6 + ax];
          } else {
            const double relx = s.atom_pos[3 * atom] - k.r[3 * e], rely = s.atom_pos[3 * atom + 1] - k.r[3 * e + 1];
            const double relz = s.atom_pos[3 * atom + 2] - k.r[3 * e + 2];
            const double dist = sqrt(relx * relx + rely * rely + relz * relz);
            const double* m = s.mesh_pts + 3 * (lane < np ? v0 + lane : v0);
            const double gx = t.R[0] * m[0] + t.R[1] * m[1] + t.R[2] * m[2];
            const double gy = t.R[3] * m[0] + t.R[4] * m[1] + t.R[5] * m[2];
            const double gz = t.R[6] * m[0] + t.R[7] * m[1] + t.R[8] * m[2];
            const double gn = sqrt(gx * gx + gy * gy + gz * gz);
            ct = (R)((-relx / dist) * (gx / gn) + (-rely / dist) * (gy / gn) + (-relz / dist) * (gz / gn));
            dmx = relx + dist * gx; dmy = rely + dist * gy; dmz = relz + dist * gz;
          }
          mx = (R)dmx; my = (R)dmy; mz = (R)dmz;
          if constexpr (kErr) {
            // the compensated form keeps the moves to FP64 accuracy: a float
            // rounding of an ECP point (about 1e-7 |r - R_I|) moves the ratio
            // by its gradient times that, which V_l near a core magnifies
            mxl = (float)(dmx - (double)mx);
            myl = (float)(dmy - (double)my);
            mzl = (float)(dmz - (double)mz);
          }
        }
      }
      R sx[P], sy[P], sz[P];
#pragma unroll
      for (int p = 0; p < P; ++p) {
        sx[p] = __shfl_sync(0xffffffffu, mx, p);
        sy[p] = __shfl_sync(0xffffffffu, my, p);
        sz[p] = __shfl_sync(0xffffffffu, mz, p);
      }
      Out ratio[P];
      float mag[P];
      // determinant locality (jqmc_gfmc.py:4980-5017): an ECP element's sign and
      // its positive (SP) value come from the determinant ratio alone, so the
      // ratio routine needs the sign of each point's weight (bit p of vneg)
      const bool dlt = kinetic && s.dlt && c >= nkc;
      unsigned vneg = 0u;
      if (dlt) {
        bool neg = false;
        if (lane < np) {
          const Out cto = (Out)ct;
          const double* vl = k.ec + (size_t)e * kEC + EC_VL;
          const Out wv = (Out)s.mesh_w[v0 + lane];
          Out vw = Out(0);
          for (int l = 0; l < s.ecp_maxl1[atom]; ++l) vw += (Out)vl[l] * (Out(2 * l + 1) * legendre_t<Out>(l, cto) * wv);
          neg = vw < Out(0);
        }
        vneg = __ballot_sync(0xffffffffu, neg);
      }
      if constexpr (kErr) {
        float sl[3 * P];
#pragma unroll
        for (int p = 0; p < P; ++p) {
          sl[p] = __shfl_sync(0xffffffffu, mxl, p);
          sl[P + p] = __shfl_sync(0xffffffffu, myl, p);
          sl[2 * P + p] = __shfl_sync(0xffffffffu, mzl, p);
        }
        wf_ratio_pts<P, R, Tab, Acc>(k, t, e, sx, sy, sz, ratio, mag, sl, dlt, vneg, lstp);
      } else {
        wf_ratio_pts<P, R, Tab, Acc>(k, t, e, sx, sy, sz, ratio, nullptr, nullptr, dlt, vneg, lstp);
      }
      if (lane < np) {
        Out rr = Out(0);
        float mg = 0.f;
#pragma unroll
        for (int p = 0; p < P; ++p) {
          rr = p == lane ? ratio[p] : rr;
          if (kErr) mg = p == lane ? mag[p] : mg;
        }
        if (c < nkc) {
          t.el[6 * e + c * P + lane] = (double)((Out)kin * rr);
          if (kErr) cancel.add(fabsf((float)kin), mg, (float)(kin * rr));
        } else {
          const int v = v0 + lane, lmax = s.ecp_maxl1[atom];
          const double* vl = k.ec + (size_t)e * kEC + EC_VL;   // V_l at the nearest nucleus
          const Out wv = (Out)s.mesh_w[v];
          const Out cto = (Out)ct;
          Out vw = Out(0);   // the element's weight: V = vw * ratio
          for (int l = 0; l < lmax; ++l) vw += (Out)vl[l] * (Out(2 * l + 1) * legendre_t<Out>(l, cto) * wv);
          // T-move: V = vw psi'/psi.  dltmove: rr is det'/det where V_det = vw det'/det
          // >= 0 and psi'/psi (the Jastrow factor, > 0, keeps the sign) elsewhere,
          // so min(V, 0) and max(V, 0) are the FN move weight and the SP part
          t.V[e * nv + v] = (double)(vw * rr);
          if (kErr) {
            cancel.add(fabsf((float)vw), mg, (float)(vw * rr));
            vmag += fabsf((float)vw) * mg;
          }
        }
      }
    }
    if constexpr (kErr) {
      vmag = warp_sum(vmag);
      if (lane == 0) t.vm[e] = vmag;
    }
  }
  __syncthreads();
  return cancel;
}

// Block energy of the mixed form: the lattice elements x_k of an electron cancel
// between the diagonal and the non-diagonal sums of E_L unless one of its six
// moves crosses a node of psi (x_k >= 0, jqmc_gfmc.py:5421-5500) and the
// fixed-node diagonal takes eu over zv = e_ion + T_e - sum_k (x_k + 1/(4a^2)).
// Only then do the float ratios reach E_L, so those electrons (a ratio below
// kFlipMargin, i.e. crossing or close enough that float rounding could decide
// the sign, and eu above zv - kFlipEnergyMargin Ha with zv from the float
// elements) get their six ratios again in FP64 arithmetic on the FP64-accurate
// tables, one warp per electron.
constexpr double kFlipMargin = 1e-3;
constexpr double kFlipEnergyMargin = 1e-2;
template <class Tab>
__device__ void refine_lattice(const Work<Tab>& k, Terms& t, double alat) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const double kin = -1.0 / (2.0 * alat * alat);
  const Sys& s = k.s;
  for (int e = wid; e < k.N; e += nw) {
    const double x = lane < 6 ? t.el[6 * e + lane] : 0.0;
    const bool near = lane < 6 && x / kin < kFlipMargin;
    if (!__any_sync(0xffffffffu, near)) continue;
    const double nd = warp_sum(lane < 6 ? x + 1.0 / (4.0 * alat * alat) : 0.0);
    const double zv = t.ei[e] + t.ke[e] - nd;
    const double eu = s.ecp_flag ? t.ei[e] : t.eid[e];
    if (!(eu > zv - kFlipEnergyMargin)) continue;   // (warp-uniform)
    for (int c = 0; c < 2; ++c) {
      double mx = 0.0, my = 0.0, mz = 0.0;
      if (lane < 3) {
        const int kk = 3 * c + lane, ax = kk >> 1;
        const double sg = (kk & 1) ? -alat : alat;
        mx = sg * t.R[ax]; my = sg * t.R[3 + ax]; mz = sg * t.R[6 + ax];
      }
      double sx[3], sy[3], sz[3], rd[3];
#pragma unroll
      for (int p = 0; p < 3; ++p) {
        sx[p] = __shfl_sync(0xffffffffu, mx, p);
        sy[p] = __shfl_sync(0xffffffffu, my, p);
        sz[p] = __shfl_sync(0xffffffffu, mz, p);
      }
      wf_ratio_pts<3, double, Tab, double>(k, t, e, sx, sy, sz, rd);
      if (lane < 3) t.el[6 * e + 3 * c + lane] = kin * (lane == 0 ? rd[0] : lane == 1 ? rd[1] : rd[2]);
    }
  }
  __syncthreads();
}

// Phase C of the GFMC_n step: (diag, nondiag) sums (jqmc_gfmc.py:4806-5030).
__device__ void lrdmc_sums(const Sys& s, const double* ec, int N, double* red, Terms& t, double alat, double* diag_out,
                           double* nondiag_out) {
  double fn = 0.0, sp = 0.0, opt = 0.0, loc = 0.0;
  for (int e = threadIdx.x; e < N; e += blockDim.x) {
    bool flip = false;
    double nd = 0.0;
    for (int kk = 0; kk < 6; ++kk) {
      const double x = t.el[6 * e + kk];
      fn += fmin(x, 0.0);
      sp += fmax(x, 0.0);
      flip = flip || (x >= 0.0);
      nd += x + 1.0 / (4.0 * alat * alat);
    }
    const double zv = t.ei[e] + t.ke[e] - nd;
    const double eu = s.ecp_flag ? t.ei[e] : t.eid[e];
    opt += flip ? fmax(zv, eu) : zv;
    loc += ec[(size_t)e * kEC + EC_ELOC];
  }
  double vfn = 0.0, vsp = 0.0;
  if (s.ecp_flag)
    for (int q = threadIdx.x; q < N * s.nv; q += blockDim.x) {
      vfn += fmin(t.V[q], 0.0);
      vsp += fmax(t.V[q], 0.0);
    }
  fn = block_sum(fn, red);
  sp = block_sum(sp, red);
  opt = block_sum(opt, red);
  vfn = block_sum(vfn, red);
  vsp = block_sum(vsp, red);
  loc = block_sum(loc, red);
  const double ee = ec[(size_t)N * kEC + EC_TOT_EE];
  const double disc = ee + s.ion_ion + opt;
  const double dk = 3.0 / (2.0 * alat * alat) * N;
  if (s.ecp_flag) {
    *nondiag_out = fn + vfn;
    *diag_out = dk + disc + loc + sp + vsp;
  } else {
    *nondiag_out = fn;
    *diag_out = dk + disc + sp;
  }
}

// ------------------------------------------------------------------ kernels
// GFMC_t arguments of k_lrdmc (tau_left == nullptr: GFMC_n)
struct TauArgs {
  double* tau_left;   // in/out, per walker
  int* nsteps;        // out: projections made in this launch
  double* eL_last;    // out: e_L of the step that spent the remaining time
};

struct KParams {
  Sys s;
  WS ws;
  TableLayout tl;
  WorkLayout wl;
  TermsLayout ml;
  int nwalk;
  int dcache_global;   // mixed form: displacement caches in ws.dcache instead of shared memory
};

__device__ __forceinline__ size_t dcache_floats_dev(const Sys& s) { return (size_t)s.N * (s.natom + s.N) * 3; }

__global__ void k_ao_vgl(Sys s, int basis, const double* __restrict__ r, long long npts, double* __restrict__ out) {
  const Basis& b = basis == 0 ? s.det : s.j3;
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= npts) return;
  const double x = r[3 * p], y = r[3 * p + 1], z = r[3 * p + 2];
  const long long nao = b.nao;
  auto f = [&](int a, double v, double gx, double gy, double gz, double lp) {
    out[(0 * nao + a) * npts + p] = v;
    out[(1 * nao + a) * npts + p] = gx;
    out[(2 * nao + a) * npts + p] = gy;
    out[(3 * nao + a) * npts + p] = gz;
    out[(4 * nao + a) * npts + p] = lp;
  };
  ao_visit_vgl<double>(b, s.atom_pos, x, y, z, f);
}

// One term of a compensated float-float dot product (algorithm Dot2 of Ogita,
// Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26 (2005)
// 1955-1988), with both factors given as float pairs x = xh + xl, y = yh + yl:
// TwoProduct (by FMA) and TwoSum are exact, so s + c carries the dot product as
// if accumulated with a 48-bit significand.  The _rn intrinsics keep the compiler
// from contracting the error-free transformations into FMAs.
__device__ __forceinline__ void dot2_step(float& s, float& c, float xh, float xl, float yh, float yl) {
  const float p = __fmul_rn(xh, yh);
  const float pe = __fmaf_rn(xh, yh, -p);
  const float t = __fadd_rn(s, p);
  const float z = __fsub_rn(t, s);
  const float se = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
  s = t;
  c += (pe + se) + fmaf(xh, yl, xl * yh);
}

// Rows of M_up = Phi_up lam (up spin) or M_dn = Phi_dn lam^T (down spin) for
// ROWS electrons per CTA, accumulated in float-float (Dot2) and stored as
// float-float pairs in the walkers' rebuild scratch: (nwalk, 2, n, A) with the M_dn block first,
// as k_walker_init reads it.  Grid (nwalk, 2 * ceil(n / ROWS)).  The AO values
// are evaluated in FP64 from the global basis tables and split into float pairs
// in shared memory (ROWS x A float2); each thread owns columns b of the output
// and reads the split lam column once per ROWS electrons.  This is the dense
// lam-GEMM of the rebuild (the geminal assembly of jqmc/determinant.py:1380-1402).
template <int ROWS>
__device__ void rebuild_m_body(const KParams& P, int w, int by, unsigned char* smem) {
  constexpr int kRebuildRows = ROWS;
  const Sys& s = P.s;
  const int n = s.n_up, A = s.det.nao;
  const int nb = (n + kRebuildRows - 1) / kRebuildRows;
  if (by >= 2 * nb) return;   // batched launches size grid.y for the largest molecule
  const int spin = by / nb, i0 = (by % nb) * kRebuildRows;
  const int rows = min(kRebuildRows, n - i0);
  float2* ph = reinterpret_cast<float2*>(smem);   // kRebuildRows x A
  const double* r = P.ws.r + ((size_t)w * s.N + (size_t)spin * s.n_up + i0) * 3;
  for (int ii = 0; ii < kRebuildRows; ++ii) {
    float2* out = ph + (size_t)ii * A;
    if (ii < rows) {
      const double px = r[3 * ii], py = r[3 * ii + 1], pz = r[3 * ii + 2];
      auto f = [&](int a, double v) {
        const float hi = (float)v;
        out[a] = make_float2(hi, (float)(v - (double)hi));
      };
      for (int sh = threadIdx.x; sh < s.det.nshell; sh += blockDim.x) {
        double dx, dy, dz;
        disp<double>(s.atom_pos, s.det.shells[kSh * sh], px, py, pz, dx, dy, dz);
        shell_val_d<double>(s.det, sh, dx, dy, dz, f);
      }
    } else {
      for (int a = threadIdx.x; a < A; a += blockDim.x) out[a] = make_float2(0.f, 0.f);
    }
  }
  __syncthreads();
  const float* __restrict__ Lh = spin == 0 ? s.lamf : s.lamTf;
  const float* __restrict__ Ll = spin == 0 ? s.laml : s.lamTl;
  // the (s, c) float-float pair is kept as it is (the value is s + c): the rest
  // of the rebuild continues in float-float
  float2* M = reinterpret_cast<float2*>(P.ws.scratch) + ((size_t)w * 2 + (spin == 0 ? 1 : 0)) * n * A + (size_t)i0 * A;
  for (int b = threadIdx.x; b < A; b += blockDim.x) {
    float sacc[kRebuildRows], cacc[kRebuildRows];
#pragma unroll
    for (int ii = 0; ii < kRebuildRows; ++ii) { sacc[ii] = 0.f; cacc[ii] = 0.f; }
#pragma unroll 2
    for (int a = 0; a < A; ++a) {
      const float yh = __ldg(Lh + (size_t)a * A + b), yl = __ldg(Ll + (size_t)a * A + b);
#pragma unroll
      for (int ii = 0; ii < kRebuildRows; ++ii) {
        const float2 x = ph[(size_t)ii * A + a];
        dot2_step(sacc[ii], cacc[ii], x.x, x.y, yh, yl);
      }
    }
#pragma unroll
    for (int ii = 0; ii < kRebuildRows; ++ii)
      if (ii < rows) M[(size_t)ii * A + b] = make_float2(sacc[ii], cacc[ii]);
  }
}

template <int ROWS>
__global__ void __launch_bounds__(128) k_rebuild_m(KParams P) {
  extern __shared__ __align__(16) unsigned char smem[];
  rebuild_m_body<ROWS>(P, blockIdx.x, blockIdx.y, smem);
}

// Operand A of the tensor-core lambda-GEMM (jqmc_tc.cu): the FP64 AO values of
// 8 electrons of one spin (rows row0 + 8 blockIdx.x + rr of the chunk; row g is
// electron g % n of walker g / n), each row scaled by 2^-e (max |phi| < 2^e) and
// split into six 8-bit integer slices, written as bf16 in the tensor cores'
// shared-memory layout: [row tile][K chunk][slice][128 x 32 canonical block].
// Rows at or past rows_total are written as zeros.  Shared memory: 8 x K doubles.
__global__ void __launch_bounds__(128) k_ao_slices(KParams P, int spin, long long row0, long long rows_total, int nk,
                                                   uint8_t* __restrict__ a_sl, int* __restrict__ row_exp,
                                                   float* __restrict__ phi_hi, float* __restrict__ phi_lo) {
  using namespace jqmc_tc;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int ex[8];
  const Sys& s = P.s;
  const int n = s.n_up, K = nk * kKC;
  double* phi = reinterpret_cast<double*>(smem);   // 8 x K
  for (int t = threadIdx.x; t < 8 * K; t += blockDim.x) phi[t] = 0.0;
  __syncthreads();
  const long long g0 = row0 + 8ll * blockIdx.x;
  for (int rr = 0; rr < 8 && g0 + rr < rows_total; ++rr) {
    const long long g = g0 + rr;
    const int w = (int)(g / n), i = (int)(g % n);
    const double* r = P.ws.r + ((size_t)w * s.N + (size_t)spin * n + i) * 3;
    const double px = r[0], py = r[1], pz = r[2];
    double* out = phi + rr * K;
    auto f = [&](int a, double v) { out[a] = v; };
    for (int sh = threadIdx.x; sh < s.det.nshell; sh += blockDim.x) {
      double dx, dy, dz;
      disp<double>(s.atom_pos, s.det.shells[kSh * sh], px, py, pz, dx, dy, dz);
      // beyond the shell's reach (e^-40) its AOs stay zero
      if ((float)(dx * dx + dy * dy + dz * dz) > __int_as_float(s.det.shells[kSh * sh + kShReach])) continue;
      shell_val_d<double>(s.det, sh, dx, dy, dz, f);
    }
  }
  __syncthreads();
  {
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int rr = wid; rr < 8; rr += blockDim.x >> 5) {
      double m = 0.0;
      for (int a = lane; a < K; a += 32) m = fmax(m, fabs(phi[rr * K + a]));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
      if (lane == 0) {
        int e = 0;
        if (m > 0.0) frexp(m, &e);
        ex[rr] = e;
      }
    }
  }
  __syncthreads();
  if (phi_hi) {
    // the rows' FP64 values as float pairs (row g = walker * n + electron, A per
    // row), which the walker initialisation reads instead of evaluating them again
    const int A = s.det.nao;
    for (int t = threadIdx.x; t < 8 * A; t += blockDim.x) {
      const int rr = t / A, a = t - rr * A;
      const long long g = g0 + rr;
      if (g >= rows_total) continue;
      const double v = phi[rr * K + a];
      const float h = (float)v;
      phi_hi[g * A + a] = h;
      phi_lo[g * A + a] = (float)(v - (double)h);
    }
  }
  const int lr0 = 8 * blockIdx.x;             // first local row of this CTA
  const int tile = lr0 / kBM, rg = (lr0 % kBM) / 8;
  if (threadIdx.x < 8) row_exp[lr0 + threadIdx.x] = ex[threadIdx.x];
  // item (k group gk of 8 AOs, row rr): the 8 lanes of consecutive rows write one
  // 128-byte core matrix per slice
  for (int it = threadIdx.x; it < 8 * (K / 8); it += blockDim.x) {
    const int rr = it & 7, gk = it >> 3;
    const double sc = ldexp(1.0, -ex[rr]);
    float q[8][kSlices];
#pragma unroll
    for (int j = 0; j < 8; ++j) split8(phi[rr * K + 8 * gk + j] * sc, q[j]);
    const int c = gk / 4;
    uint8_t* base = a_sl + ((size_t)tile * nk + c) * kAStage + rg * 512 + (gk % 4) * 128 + rr * 16;
#pragma unroll
    for (int sl = 0; sl < kSlices; ++sl) {
      unsigned short h[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) h[j] = __bfloat16_as_ushort(__float2bfloat16_rn(q[j][sl]));
      uint4 v;
      v.x = h[0] | ((unsigned)h[1] << 16);
      v.y = h[2] | ((unsigned)h[3] << 16);
      v.z = h[4] | ((unsigned)h[5] << 16);
      v.w = h[6] | ((unsigned)h[7] << 16);
      *reinterpret_cast<uint4*>(base + sl * kASliceBytes) = v;
    }
  }
}

// J3 field h_e = dJ3/dphi3(r_e) of every electron (the gradient of J3 with
// respect to one electron's J3 AO vector, jastrow_factor.py:4077-4156), with
// arithmetic type J and stored as Tab, in two passes over the electrons so that
// only four A3-vectors are held: the spin totals of phi3, then each field with
// the running prefix (the electron's J3 AO values are evaluated again).
// buf: 4 A3 values of type J.  Block-cooperative.
template <class J, class Tab>
__device__ void j3_field(const Sys& s, Tab* h, const double* r, J* buf, const J* jm, const J* jmT, float* hlo = nullptr) {
  const int N = s.N, A3 = s.j3.nao;
  J* tot_up = buf;
  J* tot_dn = buf + A3;
  J* pfx = buf + 2 * A3;
  J* pe = buf + 3 * A3;
  auto fill_phi3 = [&](int e) {
    auto f = [&](int a, J v) { pe[a] = v; };
    for (int sh = threadIdx.x; sh < s.j3.nshell; sh += blockDim.x) {
      J dx, dy, dz;
      disp<J>(s.atom_pos, s.j3.shells[kSh * sh], r[3 * e], r[3 * e + 1], r[3 * e + 2], dx, dy, dz);
      shell_val_d<J>(s.j3, sh, dx, dy, dz, f);
    }
  };
  __syncthreads();
  for (int c = threadIdx.x; c < A3; c += blockDim.x) {
    tot_up[c] = J(0);
    tot_dn[c] = J(0);
    pfx[c] = J(0);
  }
  for (int e = 0; e < N; ++e) {
    __syncthreads();
    fill_phi3(e);
    __syncthreads();
    J* tot = e < s.n_up ? tot_up : tot_dn;
    for (int c = threadIdx.x; c < A3; c += blockDim.x) tot[c] += pe[c];
  }
  for (int e = 0; e < N; ++e) {
    const bool up = e < s.n_up;
    __syncthreads();
    if (e == s.n_up)
      for (int c = threadIdx.x; c < A3; c += blockDim.x) pfx[c] = J(0);
    fill_phi3(e);
    __syncthreads();
    const J* tot_same = up ? tot_up : tot_dn;
    for (int c = threadIdx.x; c < A3; c += blockDim.x) {
      // h = j1 + J^T pfx + J (tot_same - pfx - phi_e) + (up ? J tot_dn : J^T tot_up)
      J acc = (J)s.j3vec[c];
      for (int cp = 0; cp < A3; ++cp) {
        const J Jcpc = jm[(size_t)cp * A3 + c];    // J[cp][c]
        const J Jccp = jmT[(size_t)cp * A3 + c];   // J[c][cp]
        const J pf = pfx[cp];
        acc += Jcpc * pf + Jccp * (tot_same[cp] - pf - pe[cp]);
        acc += up ? Jccp * tot_dn[cp] : Jcpc * tot_up[cp];
      }
      h[(size_t)e * A3 + c] = (Tab)acc;
      if (hlo) hlo[(size_t)e * A3 + c] = (float)((double)acc - (double)(Tab)acc);
    }
    __syncthreads();
    for (int c = threadIdx.x; c < A3; c += blockDim.x) pfx[c] += pe[c];
  }
}

// The J3 field of the mixed rebuild with the walker's rebuild scratch (free
// after the T phase) as work space, all electrons at once (j3_field's sums in
// another order and arithmetic):
//   1. phi3(r_e) of every electron in FP64 into the scratch (N x A3 doubles),
//      all (electron, shell) items;
//   2. per column c, over the electrons in order: u_e = prefix_e (+ tot_up for a
//      down electron), v_e = tot_same - prefix_e - phi3_e (+ tot_dn for an up
//      electron), prefix_e the sum of phi3 over the same-spin electrons before e,
//      in FP64 and stored as float pairs (U, V: N x A3 float2 each, over the
//      scratch);
//   3. h_e[c] = j[c] + sum_cp J[cp][c] u_e[cp] + J[c][cp] v_e[cp] for all (e, c)
//      by compensated float-float dots (Dot2) with the float pairs of J
//      (s.j3k4), a warp over 32 consecutive c of one e.
// Written in Tab with the low parts in hlo (when given).  Needs 2 N A3 doubles.
template <class Tab>
__device__ void j3_field_rows(const Sys& s, Tab* h, float* hlo, const double* r, double* scr) {
  const int N = s.N, A3 = s.j3.nao, nsh = s.j3.nshell, nu = s.n_up;
  double* Phi = scr + (size_t)N * A3;   // phase 1 output, read by phase 2 only
  float2* U = reinterpret_cast<float2*>(scr);
  float2* V = U + (size_t)N * A3;
  for (int it = threadIdx.x; it < N * nsh; it += blockDim.x) {
    const int e = it / nsh, sh = it - e * nsh;
    double* row = Phi + (size_t)e * A3;
    double dx, dy, dz;
    disp<double>(s.atom_pos, s.j3.shells[kSh * sh], r[3 * e], r[3 * e + 1], r[3 * e + 2], dx, dy, dz);
    if ((float)(dx * dx + dy * dy + dz * dz) > __int_as_float(s.j3.shells[kSh * sh + kShReach])) {
      for (int a = 0; a < s.j3.shells[kSh * sh + 5]; ++a) row[s.j3.shells[kSh * sh + 4] + a] = 0.0;
      continue;
    }
    auto f = [&](int a, double v) { row[a] = v; };
    shell_val_d<double>(s.j3, sh, dx, dy, dz, f);
  }
  __syncthreads();
  // U (float2) takes the first N A3 doubles, V the second, over Phi: element
  // (e, c) of V is written after Phi (e, c) is read, by the thread that owns
  // column c
  auto pair = [](double x) { const float hi = (float)x; return make_float2(hi, (float)(x - (double)hi)); };
  for (int c = threadIdx.x; c < A3; c += blockDim.x) {
    double tu = 0.0, td = 0.0;
    for (int e = 0; e < N; ++e) (e < nu ? tu : td) += Phi[(size_t)e * A3 + c];
    double pfx = 0.0;
    for (int e = 0; e < N; ++e) {
      if (e == nu) pfx = 0.0;
      const bool up = e < nu;
      const double phi = Phi[(size_t)e * A3 + c];
      U[(size_t)e * A3 + c] = pair(up ? pfx : pfx + tu);
      V[(size_t)e * A3 + c] = pair(up ? (tu - pfx - phi) + td : td - pfx - phi);
      pfx += phi;
    }
  }
  __syncthreads();
  for (int it = threadIdx.x; it < N * A3; it += blockDim.x) {
    const int e = it / A3, c = it - e * A3;
    const float2* u = U + (size_t)e * A3;
    const float2* v = V + (size_t)e * A3;
    float sh = 0.f, sc = 0.f;
    for (int cp = 0; cp < A3; ++cp) {
      const float4 k = s.j3k4[(size_t)cp * A3 + c];
      const float2 uu = u[cp], vv = v[cp];
      dot2_step(sh, sc, k.x, k.y, uu.x, uu.y);
      dot2_step(sh, sc, k.z, k.w, vv.x, vv.y);
    }
    const double acc = s.j3vec[c] + ((double)sh + (double)sc);
    h[it] = (Tab)acc;
    if (hlo) hlo[it] = (float)(acc - (double)(Tab)acc);
  }
}

// Walker initialisation in FP64: G, G^-1 (Gauss-Jordan, partial pivoting), T
// tables and J3 field, written in the table type Tab.  M_up / M_dn go to the
// double scratch (for Tab == double the T buffers themselves).
// mode bit 0 (kInitTablesOnly): leave the energy cache and the AO derivative
// tables alone -- they are recomputed exactly at every move, so a rebuild of a
// projected walker only needs the tables that accumulate rank-1 rounding.
// mode bit 1 (kInitRefine): one step of iterative refinement of the inverse,
// X <- X + X (I - G X), in FP64.
// mode bit 2 (kInitMReady): M_up / M_dn are already in the scratch (k_rebuild_m).
// mode bit 3 (kInitJ3Table): compute the J3 field in the table type (the float
// form's drift-control rebuild between VMC measurements; an energy is measured
// only after a full build, whose field is FP64).
// mode bit 4 (kInitPhiReady, mixed form): phi_dn of every down electron is
// already in the T buffers as float pairs (k_ao_slices).
constexpr int kInitTablesOnly = 1;
constexpr int kInitRefine = 2;
constexpr int kInitMReady = 4;
constexpr int kInitJ3Table = 8;
constexpr int kInitPhiReady = 16;
template <class Tab>
__device__ void walker_init_body(const KParams& P, int w, const InitLayout& IL, int mode,
                                 unsigned char* smem) {
  // the tables stay in global memory (read through L1): a few passes per
  // walker, and the shared memory they would take keeps a third CTA off the SM
  const Sys s = P.s;
  const int n = s.n_up, A = s.det.nao, N = s.N, A3 = s.has_j3 ? s.j3.nao : 1;
  double* r = reinterpret_cast<double*>(smem + IL.r);
  int* piv = reinterpret_cast<int*>(smem + IL.sc);
  double* Gd = reinterpret_cast<double*>(smem + IL.Gd);   // n*n
  double* aug = reinterpret_cast<double*>(smem + IL.aug); // n*2n
  double* vec = reinterpret_cast<double*>(smem + IL.vec); // max(A + n, 4*A3)
  double* vn = vec + A;                                    // n
  Tab* Tup = static_cast<Tab*>(P.ws.Tup) + (size_t)w * n * A;
  Tab* Tdn = static_cast<Tab*>(P.ws.Tdn) + (size_t)w * n * A;
  double* Mdn;  // n rows of A: row j = lambda phi_dn(r_j)
  double* Mup;  // n rows of A: row i = phi_up(r_i)^T lambda
  if constexpr (sizeof(Tab) == sizeof(double)) {
    Mdn = reinterpret_cast<double*>(Tup);
    Mup = reinterpret_cast<double*>(Tdn);
  } else {
    Mdn = P.ws.scratch + (size_t)w * 2 * n * A;
    Mup = Mdn + (size_t)n * A;
  }
  for (int t = threadIdx.x; t < N * 3; t += blockDim.x) r[t] = P.ws.r[(size_t)w * N * 3 + t];
  __syncthreads();
  const bool m_ready = (mode & kInitMReady) != 0;
  for (int i = 0; i < n && !m_ready; ++i) {
    ao_fill_block<double, double>(s.det, s.atom_pos, r[3 * i], r[3 * i + 1], r[3 * i + 2], vec);
    __syncthreads();
    for (int b = threadIdx.x; b < A; b += blockDim.x) {
      double acc = 0.0;
      for (int a = 0; a < A; ++a) acc += vec[a] * s.lam[(size_t)a * A + b];
      Mup[(size_t)i * A + b] = acc;
    }
    __syncthreads();
  }
  if constexpr (sizeof(Tab) == sizeof(float)) {
    // mixed form: M_up / M_dn are float-float pairs from k_rebuild_m (or the
    // tensor-core GEMM).  phi_dn(r_j) of every down electron in FP64, split into
    // float pairs over the T buffers (hi in T_up, lo in T_dn: free until the T
    // phase), all (electron, shell) items at once (or left there by the
    // tensor-core path's k_ao_slices: kInitPhiReady); then G[i][j] = M_up[i] .
    // phi_dn[j] by compensated float-float dots, 2 x 4 (i, j) per warp
    const float2* Mup2 = reinterpret_cast<const float2*>(Mup);
    float* ph = reinterpret_cast<float*>(Tup);
    float* pl = reinterpret_cast<float*>(Tdn);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nsh = s.det.nshell, nd = s.n_dn;
    for (int it = threadIdx.x; it < ((mode & kInitPhiReady) ? 0 : nd * nsh); it += blockDim.x) {
      const int j = it / nsh, sh = it - j * nsh, e = s.n_up + j;
      float* hi = ph + (size_t)j * A;
      float* lo = pl + (size_t)j * A;
      double dx, dy, dz;
      disp<double>(s.atom_pos, s.det.shells[kSh * sh], r[3 * e], r[3 * e + 1], r[3 * e + 2], dx, dy, dz);
      if ((float)(dx * dx + dy * dy + dz * dz) > __int_as_float(s.det.shells[kSh * sh + kShReach])) {
        for (int a = 0; a < s.det.shells[kSh * sh + 5]; ++a) {
          hi[s.det.shells[kSh * sh + 4] + a] = 0.f;
          lo[s.det.shells[kSh * sh + 4] + a] = 0.f;
        }
        continue;
      }
      auto f = [&](int a, double v) {
        const float h = (float)v;
        hi[a] = h;
        lo[a] = (float)(v - (double)h);
      };
      shell_val_d<double>(s.det, sh, dx, dy, dz, f);
    }
    __syncthreads();
    constexpr int BI = 2, BJ = 4;   // (i, j) block of one warp
    const int nbi = (n + BI - 1) / BI, nbj = (nd + BJ - 1) / BJ;
    for (int blk = wid; blk < nbi * nbj; blk += nw) {
      const int i0 = BI * (blk / nbj), j0 = BJ * (blk % nbj);
      F2 acc[BI][BJ];
#pragma unroll
      for (int u = 0; u < BI; ++u)
#pragma unroll
        for (int v = 0; v < BJ; ++v) acc_zero(acc[u][v]);
      int ri[BI], rj[BJ];
#pragma unroll
      for (int u = 0; u < BI; ++u) ri[u] = min(i0 + u, n - 1) * A;
#pragma unroll
      for (int v = 0; v < BJ; ++v) rj[v] = min(j0 + v, nd - 1) * A;
      for (int a = lane; a < A; a += 32) {
        float2 m[BI];
        float xh[BJ], xl[BJ];
#pragma unroll
        for (int u = 0; u < BI; ++u) m[u] = Mup2[ri[u] + a];
#pragma unroll
        for (int v = 0; v < BJ; ++v) { xh[v] = ph[rj[v] + a]; xl[v] = pl[rj[v] + a]; }
#pragma unroll
        for (int u = 0; u < BI; ++u)
#pragma unroll
          for (int v = 0; v < BJ; ++v) dot2_step(acc[u][v].s, acc[u][v].c, m[u].x, m[u].y, xh[v], xl[v]);
      }
#pragma unroll
      for (int u = 0; u < BI; ++u)
#pragma unroll
        for (int v = 0; v < BJ; ++v) {
          const double g = acc_out(acc[u][v]);
          if (lane == 0 && i0 + u < n && j0 + v < nd) Gd[(i0 + u) * n + j0 + v] = g;
        }
    }
    __syncthreads();
  } else {
    for (int j = 0; j < s.n_dn; ++j) {
      const int e = s.n_up + j;
      ao_fill_block<double, double>(s.det, s.atom_pos, r[3 * e], r[3 * e + 1], r[3 * e + 2], vec);
      __syncthreads();
      rows_dot<double>(Mup, n, A, vec, vn);
      for (int a = threadIdx.x; a < A && !m_ready; a += blockDim.x) {
        double acc = 0.0;
        for (int b = 0; b < A; ++b) acc += s.lamT[(size_t)b * A + a] * vec[b];
        Mdn[(size_t)j * A + a] = acc;
      }
      __syncthreads();
      for (int i = threadIdx.x; i < n; i += blockDim.x) Gd[i * n + j] = vn[i];
      __syncthreads();
    }
  }
  // Gauss-Jordan on [G | I]
  const int n2 = 2 * n;
  for (int t = threadIdx.x; t < n * n2; t += blockDim.x) {
    const int rr = t / n2, cc = t % n2;
    aug[t] = cc < n ? Gd[rr * n + cc] : (cc - n == rr ? 1.0 : 0.0);
  }
  __syncthreads();
  {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int c = 0; c < n; ++c) {
      if (wid == 0) {
        // partial pivoting: the first row of largest |G[r][c]|, r >= c (warp argmax)
        double best = -1.0;
        int p = n;
        for (int rr = c + lane; rr < n; rr += 32) {
          const double v = fabs(aug[rr * n2 + c]);
          if (v > best) { best = v; p = rr; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const double ob = __shfl_xor_sync(0xffffffffu, best, o);
          const int op = __shfl_xor_sync(0xffffffffu, p, o);
          if (ob > best || (ob == best && op < p)) { best = ob; p = op; }
        }
        if (lane == 0) {
          piv[0] = p < n ? p : c;
          if (!(best > 0.0)) atomicOr(P.ws.status + w, JQMC_ST_SINGULAR);
        }
      }
      __syncthreads();
      const int p = piv[0];
      if (p != c)
        for (int cc = threadIdx.x; cc < n2; cc += blockDim.x) {
          const double tmp = aug[c * n2 + cc];
          aug[c * n2 + cc] = aug[p * n2 + cc];
          aug[p * n2 + cc] = tmp;
        }
      __syncthreads();
      // row c / pivot; columns < c of row c are zero and column c is set to the
      // unit column below, so neither is touched here
      const double pv = aug[c * n2 + c];
      for (int cc = c + 1 + threadIdx.x; cc < n2; cc += blockDim.x) aug[c * n2 + cc] /= pv;
      __syncthreads();
      for (int rr = wid; rr < n; rr += nw) {
        if (rr == c) continue;
        const double f = aug[rr * n2 + c];
        for (int cc = c + 1 + lane; cc < n2; cc += 32) aug[rr * n2 + cc] -= f * aug[c * n2 + cc];
      }
      __syncthreads();
      for (int rr = threadIdx.x; rr < n; rr += blockDim.x) aug[rr * n2 + c] = rr == c ? 1.0 : 0.0;
      __syncthreads();
    }
  }
  Tab* Gw = static_cast<Tab*>(P.ws.G) + (size_t)w * n * n;
  Tab* Giw = static_cast<Tab*>(P.ws.Ginv) + (size_t)w * n * n;
  if (mode & kInitRefine) {
    // R = I - G X into the left half of aug (the identity left by the elimination)
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      const int rr = t / n, cc = t % n;
      double acc = rr == cc ? 1.0 : 0.0;
      for (int k = 0; k < n; ++k) acc -= Gd[rr * n + k] * aug[k * n2 + n + cc];
      aug[rr * n2 + cc] = acc;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) Gw[t] = (Tab)Gd[t];
    __syncthreads();
    // X + X R into Gd (G is written out above), then back into the right half
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      const int rr = t / n, cc = t % n;
      double acc = aug[rr * n2 + n + cc];
      for (int k = 0; k < n; ++k) acc += aug[rr * n2 + n + k] * aug[k * n2 + cc];
      Gd[t] = acc;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      aug[(t / n) * n2 + n + (t % n)] = Gd[t];
      Giw[t] = (Tab)Gd[t];
    }
  } else {
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      Gw[t] = (Tab)Gd[t];
      Giw[t] = (Tab)aug[(t / n) * n2 + n + (t % n)];
    }
  }
  __syncthreads();
  // T_up[k][a] = sum_j M_dn[j][a] G^-1[j][k] ; T_dn[k][b] = sum_i G^-1[k][i] M_up[i][b]  (per column)
  if constexpr (sizeof(Tab) == sizeof(float)) {
    // mixed form: G^-1 split into float pairs (over the G buffer, free now) and
    // compensated float-float sums, eight rows of T per pass over a column of M
    float2* Gi2 = reinterpret_cast<float2*>(Gd);
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      const double v = aug[(t / n) * n2 + n + (t % n)];
      const float hi = (float)v;
      Gi2[t] = make_float2(hi, (float)(v - (double)hi));
    }
    __syncthreads();
    const float2* Mdn2 = reinterpret_cast<const float2*>(Mdn);
    const float2* Mup2 = reinterpret_cast<const float2*>(Mup);
    float* tlo = P.ws.tlo ? P.ws.tlo + (size_t)w * tlo_stride(s) : nullptr;
    constexpr int KB = 8;
    for (int a = threadIdx.x; a < A; a += blockDim.x) {
      for (int k0 = 0; k0 < n; k0 += KB) {
        float us[KB], uc[KB], ds[KB], dc[KB];
#pragma unroll
        for (int u = 0; u < KB; ++u) { us[u] = 0.f; uc[u] = 0.f; ds[u] = 0.f; dc[u] = 0.f; }
        for (int j = 0; j < n; ++j) {
          const float2 md = Mdn2[(size_t)j * A + a], mu = Mup2[(size_t)j * A + a];
#pragma unroll
          for (int u = 0; u < KB; ++u) {
            const int kk = k0 + u < n ? k0 + u : n - 1;
            const float2 gjk = Gi2[j * n + kk], gkj = Gi2[kk * n + j];
            dot2_step(us[u], uc[u], md.x, md.y, gjk.x, gjk.y);
            dot2_step(ds[u], dc[u], gkj.x, gkj.y, mu.x, mu.y);
          }
        }
#pragma unroll
        for (int u = 0; u < KB; ++u)
          if (k0 + u < n) {
            // (s, c) -> (hi, lo) with hi the float nearest to s + c
            const float uh = __fadd_rn(us[u], uc[u]), dh = __fadd_rn(ds[u], dc[u]);
            Tup[(size_t)(k0 + u) * A + a] = (Tab)uh;
            Tdn[(size_t)(k0 + u) * A + a] = (Tab)dh;
            if (tlo) {
              tlo[(size_t)(k0 + u) * A + a] = __fadd_rn(__fsub_rn(us[u], uh), uc[u]);
              tlo[(size_t)(n + k0 + u) * A + a] = __fadd_rn(__fsub_rn(ds[u], dh), dc[u]);
            }
          }
      }
    }
  } else {
    for (int a = threadIdx.x; a < A; a += blockDim.x) {
      double m[JQMC_MAX_NUP];
      for (int j = 0; j < n; ++j) m[j] = Mdn[(size_t)j * A + a];
      for (int kk = 0; kk < n; ++kk) {
        double acc = 0.0;
        for (int j = 0; j < n; ++j) acc += m[j] * aug[j * n2 + n + kk];
        Tup[(size_t)kk * A + a] = (Tab)acc;
      }
      for (int j = 0; j < n; ++j) m[j] = Mup[(size_t)j * A + a];
      for (int kk = 0; kk < n; ++kk) {
        double acc = 0.0;
        for (int j = 0; j < n; ++j) acc += aug[kk * n2 + n + j] * m[j];
        Tdn[(size_t)kk * A + a] = (Tab)acc;
      }
    }
  }
  if (!(mode & kInitTablesOnly)) {
    // energy cache
    ecache_init(s, r, P.ws.ecache + (size_t)w * (N + 1) * kEC, reinterpret_cast<double*>(smem + IL.red));
    // AO derivative tables at every electron
    Tab* dpw = static_cast<Tab*>(P.ws.dphi) + (size_t)w * N * 4 * A;
    Tab* dp3w = s.has_j3 ? static_cast<Tab*>(P.ws.dphi3) + (size_t)w * N * 5 * A3 : nullptr;
    for (int e = 0; e < N; ++e)
      fill_dtables<Tab>(s, r[3 * e], r[3 * e + 1], r[3 * e + 2], dpw + (size_t)e * 4 * A, dp3w ? dp3w + (size_t)e * 5 * A3 : nullptr);
  }
  // J3 field, in two passes over the electrons so that only four A3-vectors are
  // held: the spin totals of phi3, then each field with the running prefix (the
  // electron's J3 AO values are evaluated again in the second pass).  In FP64
  // (the field enters every J3 ratio and the J3 gradients of the kinetic
  // energy), or in the table type with kInitJ3Table.
  if (s.has_j3) {
    Tab* h = static_cast<Tab*>(P.ws.h3) + (size_t)w * N * A3;
    // the low parts of an FP64 field go behind the T tables' in the low-part buffer
    float* hlo = sizeof(Tab) == sizeof(float) && P.ws.tlo ? P.ws.tlo + (size_t)w * tlo_stride(s) + (size_t)2 * n * A : nullptr;
    if (sizeof(Tab) == sizeof(float) && (mode & kInitJ3Table)) {
      j3_field<Tab, Tab>(s, h, r, reinterpret_cast<Tab*>(vec), j3m_of<Tab>(s), j3mT_of<Tab>(s));
      if (hlo)
        for (int c = threadIdx.x; c < N * A3; c += blockDim.x) hlo[c] = 0.f;
    } else if (sizeof(Tab) == sizeof(float) && P.ws.scratch && (size_t)2 * N * A3 <= (size_t)2 * n * A) {
      __syncthreads();   // the T phase has read the scratch
      j3_field_rows<Tab>(s, h, hlo, r, P.ws.scratch + (size_t)w * 2 * n * A);
    } else {
      j3_field<double, Tab>(s, h, r, vec, s.j3mat, s.j3matT, hlo);
    }
  }
}

template <class Tab>
__global__ void __launch_bounds__(128, 3) k_walker_init(KParams P, InitLayout IL, int mode) {
  extern __shared__ __align__(16) unsigned char smem[];
  walker_init_body<Tab>(P, blockIdx.x, IL, mode, smem);
}


// Per-walker derivatives of ln|psi| with respect to the variational parameters
// (FP64 form), the blocks grad(evaluate_ln_wavefunction) yields in the reference
// (jqmc_mcmc.py:856-876, collect_param_grads jastrow_factor.py:2110-2124 and
// determinant.py:389-399):
//   oj1[w]  d/da  of J1 = sum_{e,I} f1(a; |r_e - R_I|)       (jastrow_factor.py:649-726)
//   oj2[w]  d/db  of J2 = sum_{p<q} f2(b; r_pq)              (jastrow_factor.py:1181-1251)
//   oj3[w]  (A3, A3+1): d/dJ[a][b] = sum_{p<q same spin} phi_p[a] phi_q[b]
//           + S_up[a] S_dn[b]; last column d/dj[a] = S_up[a] + S_dn[a]   (:1744-1801)
//   olam[w] (A, A): d ln|det G| / d lambda[a][b] = sum_ij Ginv[j][i] phi_i[a] psi_j[b]
//           with G[i][j] = phi_i^T lambda psi_j (determinant.py:1380-1402)
// The AO values are recomputed from the positions (nothing is stored); the lambda
// block uses work (nwalk * 2 * n * A doubles): Phi_up rows, then X = Ginv^T Psi_dn.
// A NULL output skips its block.
__global__ void k_dlnpsi_dparam(KParams P, int off_red, int off_su, int off_sd, int off_phi3, double* oj1, double* oj2,
                                double* oj3, double* olam, double* work) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Sys& s = P.s;
  const int w = blockIdx.x;
  const int N = s.N, n = s.n_up, A = s.det.nao, M = s.natom;
  double* r = reinterpret_cast<double*>(smem);
  double* red = reinterpret_cast<double*>(smem + off_red);
  for (int t = threadIdx.x; t < N * 3; t += blockDim.x) r[t] = P.ws.r[(size_t)w * N * 3 + t];
  __syncthreads();
  if (oj1) {
    double acc = 0.0;
    if (s.has_j1) {
      const double a = s.j1_param;
      for (int t = threadIdx.x; t < N * M; t += blockDim.x) {
        const int e = t / M, at = t % M;
        const double dx = r[3 * e] - s.atom_pos[3 * at], dy = r[3 * e + 1] - s.atom_pos[3 * at + 1];
        const double dz = r[3 * e + 2] - s.atom_pos[3 * at + 2];
        const double d = sqrt(dx * dx + dy * dy + dz * dz);
        const double c = s.j1_cA[2 * at], Aa = s.j1_cA[2 * at + 1];
        if (s.j1_type == 0) {
          const double ex = exp(-a * c * d);
          acc += -Aa * (c * d * ex / (2.0 * a) - (1.0 - ex) / (2.0 * a * a));
        } else {
          const double q = 1.0 + a * c * d;
          acc += Aa * c * d * d / (2.0 * q * q);
        }
      }
    }
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) oj1[w] = acc;
  }
  if (oj2) {
    double acc = 0.0;
    if (s.has_j2) {
      const double b = s.j2_param;
      for (int t = threadIdx.x; t < N * N; t += blockDim.x) {
        const int p = t / N, q = t % N;
        if (q <= p) continue;
        const double dx = r[3 * p] - r[3 * q], dy = r[3 * p + 1] - r[3 * q + 1], dz = r[3 * p + 2] - r[3 * q + 2];
        const double d = sqrt(dx * dx + dy * dy + dz * dz);
        if (s.j2_type == 0) {
          const double u = 1.0 + b * d;
          acc += -d * d / (2.0 * u * u);
        } else {
          const double ex = exp(-b * d);
          acc += d * ex / (2.0 * b) - (1.0 - ex) / (2.0 * b * b);
        }
      }
    }
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) oj2[w] = acc;
  }
  if (oj3 && s.has_j3) {
    const int A3 = s.j3.nao, nsh = s.j3.nshell;
    double* su = reinterpret_cast<double*>(smem + off_su);
    double* sd = reinterpret_cast<double*>(smem + off_sd);
    double* phi3 = reinterpret_cast<double*>(smem + off_phi3);   // N x A3
    for (int t = threadIdx.x; t < N * nsh; t += blockDim.x) {
      const int e = t / nsh, sh = t % nsh;
      double* out = phi3 + (size_t)e * A3;
      auto f = [&](int a, double v) { out[a] = v; };
      double dx, dy, dz;
      disp<double>(s.atom_pos, s.j3.shells[kSh * sh], r[3 * e], r[3 * e + 1], r[3 * e + 2], dx, dy, dz);
      shell_val_d<double>(s.j3, sh, dx, dy, dz, f);
    }
    __syncthreads();
    for (int a = threadIdx.x; a < A3; a += blockDim.x) {
      double tu = 0.0, td = 0.0;
      for (int e = 0; e < n; ++e) tu += phi3[(size_t)e * A3 + a];
      for (int e = n; e < N; ++e) td += phi3[(size_t)e * A3 + a];
      su[a] = tu;
      sd[a] = td;
    }
    __syncthreads();
    double* o = oj3 + (size_t)w * A3 * (A3 + 1);
    for (int t = threadIdx.x; t < A3 * A3; t += blockDim.x) {
      const int a = t / A3, b = t % A3;
      double acc = su[a] * sd[b];
      for (int sp = 0; sp < 2; ++sp) {
        double pa = 0.0;
        for (int q = sp * n; q < (sp + 1) * n; ++q) {
          acc += pa * phi3[(size_t)q * A3 + b];
          pa += phi3[(size_t)q * A3 + a];
        }
      }
      o[(size_t)a * (A3 + 1) + b] = acc;
    }
    for (int a = threadIdx.x; a < A3; a += blockDim.x) o[(size_t)a * (A3 + 1) + A3] = su[a] + sd[a];
    __syncthreads();
  }
  if (olam) {
    const int nsh = s.det.nshell;
    double* Phi = work + (size_t)w * 2 * n * A;
    double* X = Phi + (size_t)n * A;
    for (int t = threadIdx.x; t < 2 * n * nsh; t += blockDim.x) {
      const int e = t / nsh, sh = t % nsh;   // e < n: up electron e (Phi row); else down electron e - n (X row)
      double* out = e < n ? Phi + (size_t)e * A : X + (size_t)(e - n) * A;
      auto f = [&](int a, double v) { out[a] = v; };
      double dx, dy, dz;
      disp<double>(s.atom_pos, s.det.shells[kSh * sh], r[3 * e], r[3 * e + 1], r[3 * e + 2], dx, dy, dz);
      shell_val_d<double>(s.det, sh, dx, dy, dz, f);
    }
    __syncthreads();
    const double* Gi = static_cast<const double*>(P.ws.Ginv) + (size_t)w * n * n;
    for (int b = threadIdx.x; b < A; b += blockDim.x) {
      double col[JQMC_MAX_NUP];
      for (int j = 0; j < n; ++j) col[j] = X[(size_t)j * A + b];
      for (int i = 0; i < n; ++i) {
        double acc = 0.0;
        for (int j = 0; j < n; ++j) acc += Gi[j * n + i] * col[j];
        X[(size_t)i * A + b] = acc;
      }
    }
    __syncthreads();
    double* o = olam + (size_t)w * A * A;
    for (long long t = threadIdx.x; t < (long long)A * A; t += blockDim.x) {
      const int a = (int)(t / A), b = (int)(t % A);
      double acc = 0.0;
      for (int i = 0; i < n; ++i) acc += Phi[(size_t)i * A + a] * X[(size_t)i * A + b];
      o[t] = acc;
    }
  }
}

// d ln|psi| / dR_I for every nucleus I (FP64 walkers), the Pulay part of the
// force (force_PP of jqmc_mcmc.py:780-845 without space warp).  Every AO sits
// on a nucleus, d phi_a(r - R_I)/dR_I = -grad phi_a, so the derivative is minus
// each electron's grad ln psi restricted to the AOs on I: geminal AOs through
// the T rows (grad ln det_e = sum_a grad phi_a(r_e) T_e[a]), J3 AOs through the
// J3 field, and the J1 pair terms.  Reads the walker's cached derivative tables;
// out: nwalk x natom x 3.
__global__ void k_dlnpsi_dR(KParams P, int off_acc, double* out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int w = blockIdx.x;
  const Sys s = stage_tables(P.s, P.tl, smem);
  Work<double> k = make_work<double>(s, P.wl, smem, P.ws, w);
  load_walker(k, P.ws, w);
  const int N = k.N, n = k.n, A = k.A, M = s.natom;
  double* acc = reinterpret_cast<double*>(smem + off_acc);   // M x 3
  for (int t = threadIdx.x; t < 3 * M; t += blockDim.x) acc[t] = 0.0;
  __syncthreads();
  const int nsh = s.det.nshell;
  for (int p = threadIdx.x; p < N * nsh; p += blockDim.x) {
    const int e = p / nsh, sh = p % nsh;
    const int* row = s.det.shells + kSh * sh;
    const int atom = row[0], ao0 = row[4], nm = row[5];
    const double* T = (e < n ? k.Tup + (size_t)e * A : k.Tdn + (size_t)(e - n) * A);
    const double* dp = k.dphi + (size_t)e * 4 * A;
    double gx = 0.0, gy = 0.0, gz = 0.0;
    for (int a = ao0; a < ao0 + nm; ++a) {
      gx += dp[a] * T[a];
      gy += dp[A + a] * T[a];
      gz += dp[2 * A + a] * T[a];
    }
    atomicAdd(acc + 3 * atom, -gx);
    atomicAdd(acc + 3 * atom + 1, -gy);
    atomicAdd(acc + 3 * atom + 2, -gz);
  }
  if (s.has_j3) {
    const int A3 = k.A3, nsh3 = s.j3.nshell;
    for (int p = threadIdx.x; p < N * nsh3; p += blockDim.x) {
      const int e = p / nsh3, sh = p % nsh3;
      const int* row = s.j3.shells + kSh * sh;
      const int atom = row[0], ao0 = row[4], nm = row[5];
      const double* h = k.h3 + (size_t)e * A3;
      const double* q = k.dphi3 + (size_t)e * 5 * A3;
      double gx = 0.0, gy = 0.0, gz = 0.0;
      for (int c = ao0; c < ao0 + nm; ++c) {
        gx += q[A3 + c] * h[c];
        gy += q[2 * A3 + c] * h[c];
        gz += q[3 * A3 + c] * h[c];
      }
      atomicAdd(acc + 3 * atom, -gx);
      atomicAdd(acc + 3 * atom + 1, -gy);
      atomicAdd(acc + 3 * atom + 2, -gz);
    }
  }
  if (s.has_j1) {
    const double aa = s.j1_param;
    for (int p = threadIdx.x; p < N * M; p += blockDim.x) {
      const int e = p / M, at = p % M;
      const double dx = k.r[3 * e] - s.atom_pos[3 * at], dy = k.r[3 * e + 1] - s.atom_pos[3 * at + 1];
      const double dz = k.r[3 * e + 2] - s.atom_pos[3 * at + 2];
      const double d = sqrt(dx * dx + dy * dy + dz * dz);
      const double c = s.j1_cA[2 * at], AA = s.j1_cA[2 * at + 1];
      double f1;   // d f1 / d |r - R|
      if (s.j1_type == 0) {
        f1 = -AA * c * exp(-aa * c * d) / 2.0;
      } else {
        const double q = 1.0 + aa * c * d;
        f1 = -AA / (2.0 * q * q);
      }
      atomicAdd(acc + 3 * at, -f1 * dx / d);
      atomicAdd(acc + 3 * at + 1, -f1 * dy / d);
      atomicAdd(acc + 3 * at + 2, -f1 * dz / d);
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < 3 * M; t += blockDim.x) out[(size_t)w * 3 * M + t] = acc[t];
}

// ln|det G|, sign (LU with partial pivoting on a copy of G) and J   (FP64 form)
// Per-electron derivatives of ln|psi| and kinetic elements (FP64 walkers), from
// the AO derivative tables, the T rows, the J3 field and the energy cache:
// out[(w N + e) 9 + (0..2)] d ln|det| / dr_e, [3] lap_e ln|det|, [4..6] dJ / dr_e,
// [7] lap_e J, [8] T_e = -1/2 (lap_e ln psi + |grad_e ln psi|^2)
// (determinant.py:1809-1900, jastrow_factor.py:2983-3060, wavefunction.py:1081-1140).
// One warp per electron.
__global__ void k_electron_terms(KParams P, double* out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int w = blockIdx.x;
  const Sys s = stage_tables(P.s, P.tl, smem);
  Work<double> k = make_work<double>(s, P.wl, smem, P.ws, w);
  load_walker(k, P.ws, w);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int A = k.A, A3 = k.A3;
  for (int e = wid; e < k.N; e += nw) {
    const bool up = e < s.n_up;
    const int i = up ? e : e - s.n_up;
    const double* Trow = (up ? k.Tup : k.Tdn) + (size_t)i * A;
    const double* dp = k.dphi + (size_t)e * 4 * A;
    double gx = 0.0, gy = 0.0, gz = 0.0, lp = 0.0, hx = 0.0, hy = 0.0, hz = 0.0, hl = 0.0;
    for (int a = lane; a < A; a += 32) {
      const double tv = Trow[a];
      gx += dp[a] * tv;
      gy += dp[A + a] * tv;
      gz += dp[2 * A + a] * tv;
      lp += dp[3 * A + a] * tv;
    }
    if (s.has_j3) {
      const double* h = k.h3 + (size_t)e * A3;
      const double* q = k.dphi3 + (size_t)e * 5 * A3;
      for (int a = lane; a < A3; a += 32) {
        const double hv = h[a];
        hx += q[A3 + a] * hv;
        hy += q[2 * A3 + a] * hv;
        hz += q[3 * A3 + a] * hv;
        hl += q[4 * A3 + a] * hv;
      }
    }
    gx = warp_sum(gx); gy = warp_sum(gy); gz = warp_sum(gz); lp = warp_sum(lp);
    hx = warp_sum(hx); hy = warp_sum(hy); hz = warp_sum(hz); hl = warp_sum(hl);
    if (lane == 0) {
      const double* row = k.ec + (size_t)e * kEC;
      const double jx = hx + row[EC_J1G] + row[EC_J2G];
      const double jy = hy + row[EC_J1G + 1] + row[EC_J2G + 1];
      const double jz = hz + row[EC_J1G + 2] + row[EC_J2G + 2];
      const double jl = hl + row[EC_J1L] + row[EC_J2L];
      const double dl = lp - (gx * gx + gy * gy + gz * gz);
      const double Gx = gx + jx, Gy = gy + jy, Gz = gz + jz;
      double* o = out + ((size_t)w * k.N + e) * 9;
      o[0] = gx; o[1] = gy; o[2] = gz; o[3] = dl;
      o[4] = jx; o[5] = jy; o[6] = jz; o[7] = jl;
      o[8] = -0.5 * (dl + jl + Gx * Gx + Gy * Gy + Gz * Gz);
    }
  }
}

// Discretised kinetic elements of every electron's six rotated lattice moves
// (FP64 walkers): out[(w N + e) 6 + k] = -psi(r_e + a s_k)/psi / (2 a^2), with
// s_k = +-column k/2 of R(angles[w]) in the order +x, -x, +y, -y, +z, -z
// (wavefunction.py:1620-1740).
__global__ void k_kinetic_mesh(KParams P, const double* __restrict__ angles, double alat, double* out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int w = blockIdx.x;
  const Sys s = stage_tables(P.s, P.tl, smem);
  Work<double> k = make_work<double>(s, P.wl, smem, P.ws, w);
  Terms t = make_terms(P.ml, smem, nullptr, s);
  load_walker(k, P.ws, w);
  if (threadIdx.x == 0) rotation(angles[3 * w], angles[3 * w + 1], angles[3 * w + 2], t.R);
  __syncthreads();
  electron_terms<double, double>(k, t, alat);
  mesh_terms<double, double, double>(k, t, alat, true);
  for (int q = threadIdx.x; q < 6 * k.N; q += blockDim.x) out[(size_t)w * 6 * k.N + q] = t.el[q];
}

__global__ void k_log_psi(KParams P, int off_aug, double* logdet, double* sign, double* jas) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int w = blockIdx.x;
  const Sys s = stage_tables(P.s, P.tl, smem);
  Work<double> k = make_work<double>(s, P.wl, smem, P.ws, w);
  load_walker(k, P.ws, w);
  const int n = k.n, N = k.N;
  double* a = reinterpret_cast<double*>(smem + off_aug);
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) a[t] = k.G[t];
  __syncthreads();
  if (threadIdx.x == 0) {
    double ld = 0.0, sg = 1.0;
    for (int c = 0; c < n; ++c) {
      int p = c;
      double best = fabs(a[c * n + c]);
      for (int rr = c + 1; rr < n; ++rr)
        if (fabs(a[rr * n + c]) > best) { best = fabs(a[rr * n + c]); p = rr; }
      if (p != c) {
        sg = -sg;
        for (int cc = 0; cc < n; ++cc) { const double tmp = a[c * n + cc]; a[c * n + cc] = a[p * n + cc]; a[p * n + cc] = tmp; }
      }
      const double pv = a[c * n + c];
      if (pv < 0) sg = -sg;
      ld += log(fabs(pv));
      for (int rr = c + 1; rr < n; ++rr) {
        const double f = a[rr * n + c] / pv;
        for (int cc = c + 1; cc < n; ++cc) a[rr * n + cc] -= f * a[c * n + cc];
      }
    }
    logdet[w] = ld;
    sign[w] = sg;
  }
  // J = J1 + J2 + J3;  J3 = (sum_e phi3_e . h_e + j1 . sum_e phi3_e) / 2
  double j = 0.0;
  for (int e = threadIdx.x; e < N; e += blockDim.x) {
    const double x = k.r[3 * e], y = k.r[3 * e + 1], z = k.r[3 * e + 2];
    if (s.has_j1) j += j1_at<double>(s, x, y, z);
    if (s.has_j2) j += 0.5 * j2_at<double>(s, k.r, e, x, y, z);
    if (s.has_j3) {
      const double* h = k.h3 + (size_t)e * k.A3;
      double acc = 0.0;
      auto f = [&](int aa, double v) { acc += v * (h[aa] + s.j3vec[aa]); };
      ao_visit<double>(s.j3, s.atom_pos, x, y, z, f);
      j += 0.5 * acc;
    }
  }
  j = block_sum(j, k.red);
  if (threadIdx.x == 0) jas[w] = j;
}

template <class Tab>
__device__ double as_factor_block(const Work<Tab>& k) {
  const int n = k.n;
  Tab F = Tab(0);
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) F += k.Gi[t] * k.Gi[t];
  const double Fs = block_sum((double)F, k.red);
  double mn = 1e300;
  for (int t = threadIdx.x; t < 2 * n; t += blockDim.x) {
    Tab acc = Tab(0);
    if (t < n) for (int c = 0; c < n; ++c) acc += k.G[t * n + c] * k.G[t * n + c];
    else for (int rr = 0; rr < n; ++rr) acc += k.G[rr * n + (t - n)] * k.G[rr * n + (t - n)];
    mn = fmin(mn, (double)acc);
  }
  mn = block_min(mn, k.red);
  const double SF = mn * Fs;
  return SF > 0.0 ? pow(SF, -3.0 / 8.0) : 0.0;
}

// VMC: K Metropolis proposals per walker (jqmc_mcmc.py:4316-4523)
// Mixed form: the proposal of one step computed by warp 0 in float, lanes over
// nuclei (jqmc_mcmc.py:4340-4400): nearest nucleus of the old and the new
// position, the f_l step scale, the Gaussian move along one axis (positions in
// double), the transition ratio and the J1 difference as a sum of pair
// differences; writes k.sc[0..5] as the FP64 code does.  The same float f_l
// values scale the move and enter the ratio, so the proposal densities stay
// consistent.
template <class Tab>
__device__ void vmc_propose_warp(Work<Tab>& k, const Sys& s, const int* id, const double* fd, double Dt) {
  const int lane = threadIdx.x & 31;
  const int e = id[0] < s.n_up ? id[1] : s.n_up + id[2];
  const double ox = k.r[3 * e], oy = k.r[3 * e + 1], oz = k.r[3 * e + 2];
  auto nearest = [&](float sx, float sy, float sz, int& best, float& bd) {
    bd = 3.0e38f;
    best = 0x7fffffff;
    for (int a = lane; a < s.natom; a += 32) {
      const float dx = (float)(ox - s.atom_pos[3 * a]) + sx, dy = (float)(oy - s.atom_pos[3 * a + 1]) + sy;
      const float dz = (float)(oz - s.atom_pos[3 * a + 2]) + sz;
      const float d = sqrtf(dx * dx + dy * dy + dz * dz);
      if (d < bd) { bd = d; best = a; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float od = __shfl_xor_sync(0xffffffffu, bd, o);
      const int ob = __shfl_xor_sync(0xffffffffu, best, o);
      if (od < bd || (od == bd && ob < best)) { bd = od; best = ob; }
    }
  };
  auto fscale = [&](int a, float d) {
    const float Z = (float)s.atom_zeff[a];
    return 1.0f / (Z * Z) * (1.0f + Z * Z * d) / (1.0f + d);
  };
  int ao;
  float dao;
  nearest(0.f, 0.f, 0.f, ao, dao);
  const float fl = fscale(ao, dao);
  const float g = (float)fd[0] * (fl * (float)Dt);
  const int ax = id[3];
  const float mx = ax == 0 ? g : 0.f, my = ax == 1 ? g : 0.f, mz = ax == 2 ? g : 0.f;
  int an;
  float dan;
  nearest(mx, my, mz, an, dan);
  const float fp = fscale(an, dan);
  const float dtf = (float)Dt;
  const float d2 = g * g;
  const float Tr = (fl / fp) * expf(-d2 * (1.0f / (2.0f * fp * fp * dtf * dtf) - 1.0f / (2.0f * fl * fl * dtf * dtf)));
  float dj = 0.f;
  if (s.has_j1) {
    const float a = (float)s.j1_param;
    for (int at = lane; at < s.natom; at += 32) {
      const float dx = (float)(ox - s.atom_pos[3 * at]), dy = (float)(oy - s.atom_pos[3 * at + 1]);
      const float dz = (float)(oz - s.atom_pos[3 * at + 2]);
      dj += pair_delta<float, true>(dx, dy, dz, mx, my, mz, s.j1_type, a, (float)s.j1_cA[2 * at], (float)s.j1_cA[2 * at + 1],
                                    true);
    }
    dj = warp_sum(dj);
  }
  if (lane == 0) {
    k.sc[0] = e;
    k.sc[1] = ox + (double)mx; k.sc[2] = oy + (double)my; k.sc[3] = oz + (double)mz;
    k.sc[4] = (double)Tr;
    k.sc[5] = (double)dj;
  }
}

// proposal selection, f_l-scaled Gaussian move and T ratio in double on
// thread 0; the determinant ratio from the T row, the candidate G^-1 / G for the
// AS factor and the accepted rank-1 update in the table type Tab; J1/J2/J3
// differences and the acceptance in double.  caches == 0: the AO derivative
// tables and the energy cache are not kept current (they are rebuilt by
// jqmc_walker_init before an energy is measured).
template <class Tab, bool CACHES>
__device__ void vmc_sweep_body(const KParams& P, int w, int K, const int* __restrict__ idraw, const double* __restrict__ fdraw,
                               double Dt, double eps_AS, int* accept, int off_cand, unsigned char* smem) {
  const Sys s = stage_tables(P.s, P.tl, smem);
  Work<Tab> k = make_work<Tab>(s, P.wl, smem, P.ws, w);
  load_walker(k, P.ws, w);
  const int n = k.n, A = k.A, A3 = k.A3;
  Tab* cand = reinterpret_cast<Tab*>(smem + off_cand);  // n*n candidate G^-1
  Tab* Gc = cand + n * n;                                // n*n candidate G
  int nacc = 0;
  double R_old = as_factor_block(k);
  for (int step = 0; step < K; ++step) {
    const int* id = idraw + ((size_t)w * K + step) * 4;
    const double* fd = fdraw + ((size_t)w * K + step) * 2;
    if constexpr (sizeof(Tab) == sizeof(float)) {
      if (threadIdx.x < 32) vmc_propose_warp<Tab>(k, s, id, fd, Dt);
    } else if (threadIdx.x == 0) {
      const int sel = id[0];
      const bool is_up = sel < s.n_up;
      const int e = is_up ? id[1] : s.n_up + id[2];
      const double ox = k.r[3 * e], oy = k.r[3 * e + 1], oz = k.r[3 * e + 2];
      int a0 = nearest_atom(s, ox, oy, oz);
      double Z = s.atom_zeff[a0];
      double dd = sqrt((ox - s.atom_pos[3 * a0]) * (ox - s.atom_pos[3 * a0]) + (oy - s.atom_pos[3 * a0 + 1]) * (oy - s.atom_pos[3 * a0 + 1]) +
                       (oz - s.atom_pos[3 * a0 + 2]) * (oz - s.atom_pos[3 * a0 + 2]));
      const double fl = 1.0 / (Z * Z) * (1.0 + Z * Z * dd) / (1.0 + dd);
      const double g = fd[0] * (fl * Dt);
      double nx = ox, ny = oy, nz = oz;
      if (id[3] == 0) nx += g; else if (id[3] == 1) ny += g; else nz += g;
      a0 = nearest_atom(s, nx, ny, nz);
      Z = s.atom_zeff[a0];
      dd = sqrt((nx - s.atom_pos[3 * a0]) * (nx - s.atom_pos[3 * a0]) + (ny - s.atom_pos[3 * a0 + 1]) * (ny - s.atom_pos[3 * a0 + 1]) +
                (nz - s.atom_pos[3 * a0 + 2]) * (nz - s.atom_pos[3 * a0 + 2]));
      const double fp = 1.0 / (Z * Z) * (1.0 + Z * Z * dd) / (1.0 + dd);
      const double d2 = (nx - ox) * (nx - ox) + (ny - oy) * (ny - oy) + (nz - oz) * (nz - oz);
      const double Tr = (fl / fp) * exp(-d2 * (1.0 / (2.0 * fp * fp * Dt * Dt) - 1.0 / (2.0 * fl * fl * Dt * Dt)));
      k.sc[0] = e;
      k.sc[1] = nx; k.sc[2] = ny; k.sc[3] = nz;
      k.sc[4] = Tr;
      double dJ = 0.0;
      if (s.has_j1) dJ += j1_at<double>(s, nx, ny, nz) - j1_at<double>(s, ox, oy, oz);
      k.sc[5] = dJ;
    }
    __syncthreads();
    const int e = (int)k.sc[0];
    const double nx = k.sc[1], ny = k.sc[2], nz = k.sc[3];
    const bool up = e < s.n_up;
    const int i = up ? e : e - s.n_up;
    double dJ = 0.0;
    if (s.has_j2) {
      if constexpr (sizeof(Tab) == sizeof(float)) {
        // pair differences from the float displacement r_e - r_m and the move
        const float sx = (float)(nx - k.r[3 * e]), sy = (float)(ny - k.r[3 * e + 1]), sz = (float)(nz - k.r[3 * e + 2]);
        const float b = (float)s.j2_param;
        float dj2 = 0.f;
        for (int m = threadIdx.x; m < k.N; m += blockDim.x) {
          if (m == e) continue;
          const float dx = (float)(k.r[3 * e] - k.r[3 * m]), dy = (float)(k.r[3 * e + 1] - k.r[3 * m + 1]);
          const float dz = (float)(k.r[3 * e + 2] - k.r[3 * m + 2]);
          dj2 += pair_delta<float, true>(dx, dy, dz, sx, sy, sz, s.j2_type, b, 0.f, 0.f, false);
        }
        dJ = (double)dj2;
      } else {
        for (int m = threadIdx.x; m < k.N; m += blockDim.x) {
          if (m == e) continue;
          const double ax = nx - k.r[3 * m], ay = ny - k.r[3 * m + 1], az = nz - k.r[3 * m + 2];
          const double bx = k.r[3 * e] - k.r[3 * m], by = k.r[3 * e + 1] - k.r[3 * m + 1], bz = k.r[3 * e + 2] - k.r[3 * m + 2];
          dJ += j2_pair<double>(s.j2_type, s.j2_param, sqrt(ax * ax + ay * ay + az * az)) -
                j2_pair<double>(s.j2_type, s.j2_param, sqrt(bx * bx + by * by + bz * bz));
        }
      }
    }
    ao_fill_block<Tab, Tab>(s.det, s.atom_pos, nx, ny, nz, k.vA0);
    if (s.has_j3) {
      ao_fill_block<Tab, Tab>(s.j3, s.atom_pos, nx, ny, nz, k.v30);
      ao_fill_block<Tab, Tab>(s.j3, s.atom_pos, k.r[3 * e], k.r[3 * e + 1], k.r[3 * e + 2], k.v31);
    }
    __syncthreads();
    if (s.has_j3) {
      Tab d3 = Tab(0);
      for (int a = threadIdx.x; a < A3; a += blockDim.x) d3 += (k.v30[a] - k.v31[a]) * k.h3[(size_t)e * A3 + a];
      dJ += (double)d3;
    }
    dJ = block_sum(dJ, k.red);
    rows_dot<Tab>(up ? k.Tup : k.Tdn, n, A, k.vA0, k.vn0);
    __syncthreads();
    const Tab ratio = k.vn0[i];
    const Tab inv = Tab(1) / ratio;
    if (up) {
      for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
        const int rr = t / n, cc = t % n;
        cand[t] = k.Gi[t] - k.Gi[rr * n + i] * (k.vn0[cc] - (cc == i ? Tab(1) : Tab(0))) * inv;
        if (rr == i) {
          Tab g = Tab(0);
          for (int q = 0; q < n; ++q) g += k.vn0[q] * k.G[q * n + cc];
          Gc[t] = g;
        } else {
          Gc[t] = k.G[t];
        }
      }
    } else {
      for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
        const int rr = t / n, cc = t % n;
        cand[t] = k.Gi[t] - (k.vn0[rr] - (rr == i ? Tab(1) : Tab(0))) * k.Gi[i * n + cc] * inv;
        if (cc == i) {
          Tab g = Tab(0);
          for (int q = 0; q < n; ++q) g += k.G[rr * n + q] * k.vn0[q];
          Gc[t] = g;
        } else {
          Gc[t] = k.G[t];
        }
      }
    }
    __syncthreads();
    Tab Fp = Tab(0);
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) Fp += cand[t] * cand[t];
    const double F = block_sum((double)Fp, k.red);
    double mn = 1e300;
    for (int t = threadIdx.x; t < 2 * n; t += blockDim.x) {
      Tab acc = Tab(0);
      if (t < n) for (int c = 0; c < n; ++c) acc += Gc[t * n + c] * Gc[t * n + c];
      else for (int rr = 0; rr < n; ++rr) acc += Gc[rr * n + (t - n)] * Gc[rr * n + (t - n)];
      mn = fmin(mn, (double)acc);
    }
    mn = block_min(mn, k.red);
    const double SF = mn * F;
    double R_new = 0.0;   // only thread 0 decides, so only it evaluates the power
    if (threadIdx.x == 0) {
      if constexpr (sizeof(Tab) == sizeof(float)) {
        const float Rn = SF > 0.0 ? powf((float)SF, -0.375f) : 0.f;
        const float Ro = (float)R_old, ea = (float)eps_AS;
        const float Jr = expf((float)(k.sc[5] + dJ));
        const float Ras = (fmaxf(Rn, ea) / Rn) / (fmaxf(Ro, ea) / Ro);
        const float x = Ras * Jr * (float)ratio;
        const float pacc = fminf(1.0f, x * x * (float)k.sc[4]);
        k.sc[6] = (fd[1] < (double)pacc) ? 1.0 : 0.0;
        R_new = (double)Rn;
      } else {
        R_new = SF > 0.0 ? pow(SF, -3.0 / 8.0) : 0.0;
        const double Jr = exp(k.sc[5] + dJ);
        const double Ras = (fmax(R_new, eps_AS) / R_new) / (fmax(R_old, eps_AS) / R_old);
        const double Rr = pow(Ras * Jr * (double)ratio, 2.0);
        const double pacc = fmin(1.0, Rr * k.sc[4]);
        k.sc[6] = (fd[1] < pacc) ? 1.0 : 0.0;
      }
    }
    __syncthreads();
    if (k.sc[6] != 0.0) {
      sm_move<Tab, CACHES>(k, e, nx, ny, nz);
      R_old = R_new;
      ++nacc;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) accept[w] += nacc;
  store_walker(k, P.ws, w);
}

__global__ void k_vmc_sweep(KParams P, int K, const int* __restrict__ idraw, const double* __restrict__ fdraw, double Dt,
                            double eps_AS, int* accept, int off_cand) {
  extern __shared__ __align__(16) unsigned char smem[];
  vmc_sweep_body<double, true>(P, blockIdx.x, K, idraw, fdraw, Dt, eps_AS, accept, off_cand, smem);
}

// ------------------------------------------------------------------ batches of systems
// One launch over the walkers of many systems (molecules): item i owns walkers
// [woff[i], woff[i+1]) of the batch; each CTA finds its item by binary search
// and runs the single-system body with that item's parameters.
struct BatchItem {
  KParams P;
  int woff;        // first walker of the item in the batch
  int off_cand;    // VMC sweep: candidate G^-1 / G offset in shared memory
  InitLayout init; // shared-memory layout of the rebuild
};

__device__ __forceinline__ int batch_item(const int* __restrict__ woff, int nitem, int g) {
  int lo = 0, hi = nitem - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (woff[mid] <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <class Tab, bool CACHES>
__global__ void k_vmc_sweep_batch(const BatchItem* __restrict__ items, const int* __restrict__ woff, int nitem, int K,
                                  const int* __restrict__ idraw, const double* __restrict__ fdraw, double Dt, double eps_AS,
                                  int* accept) {
  extern __shared__ __align__(16) unsigned char smem[];
  const BatchItem& it = items[batch_item(woff, nitem, blockIdx.x)];
  const size_t g0 = (size_t)it.woff;
  vmc_sweep_body<Tab, CACHES>(it.P, blockIdx.x - it.woff, K, idraw + g0 * K * 4, fdraw + g0 * K * 2, Dt, eps_AS, accept + g0,
                              it.off_cand, smem);
}

template <int ROWS>
__global__ void __launch_bounds__(128) k_rebuild_m_batch(const BatchItem* __restrict__ items, const int* __restrict__ woff,
                                                         int nitem) {
  extern __shared__ __align__(16) unsigned char smem[];
  const BatchItem& it = items[batch_item(woff, nitem, blockIdx.x)];
  rebuild_m_body<ROWS>(it.P, blockIdx.x - it.woff, blockIdx.y, smem);
}

template <class Tab>
__global__ void k_walker_init_batch(const BatchItem* __restrict__ items, const int* __restrict__ woff, int nitem, int mode) {
  extern __shared__ __align__(16) unsigned char smem[];
  const BatchItem& it = items[batch_item(woff, nitem, blockIdx.x)];
  walker_init_body<Tab>(it.P, blockIdx.x - it.woff, it.init, mode, smem);
}

// VMC local energy and weight (hamiltonians.py:225-290, jqmc_mcmc.py:725-747)   (FP64 form)
__global__ void k_vmc_measure(KParams P, const double* __restrict__ angles, double eps_AS, double* eL, double* wL) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int w = blockIdx.x;
  const Sys s = stage_tables(P.s, P.tl, smem);
  Work<double> k = make_work<double>(s, P.wl, smem, P.ws, w);
  Terms t = make_terms(P.ml, smem, nullptr, s);
  load_walker(k, P.ws, w);
  if (threadIdx.x == 0) rotation(angles[3 * w], angles[3 * w + 1], angles[3 * w + 2], t.R);
  __syncthreads();
  electron_terms<double>(k, t, 0.0);
  mesh_terms<double, double>(k, t, 0.0, false);
  double acc = 0.0;
  for (int e = threadIdx.x; e < k.N; e += blockDim.x) acc += t.ke[e] + t.ei[e] + k.ec[(size_t)e * kEC + EC_ELOC];
  if (s.ecp_flag)
    for (int q = threadIdx.x; q < k.N * s.nv; q += blockDim.x) acc += t.V[q];
  acc = block_sum(acc, k.red);
  const double ee = k.ec[(size_t)k.N * kEC + EC_TOT_EE];
  const double loc = 0.0;
  const double R = as_factor_block(k);
  if (threadIdx.x == 0) {
    eL[w] = acc + ee + s.ion_ion + loc;
    const double q = R / fmax(R, eps_AS);
    wL[w] = q * q;
  }
}

// LRDMC GFMC_n projections; K steps fused.  K == 0 with energy outputs computes
// e_L and V_diag at the current positions with the rotation of draw[w].
// R: mesh arithmetic, Tab: table storage and updates.
// Block-energy modes of k_lrdmc (mixed form): kEnergyBound writes the walker's
// cancellation factor C of the compensated-float energy to the first double of
// its rebuild scratch (free after the rebuild); kEnergyGate runs only the
// walkers whose C exceeds kFastEnergyCancel and overwrites their energy.
constexpr int kEnergyPlain = 0, kEnergyBound = 1, kEnergyGate = 2;
constexpr double kFastEnergyCancel = JQMC_FAST_ENERGY_CANCEL;
__device__ __forceinline__ double* energy_bound(const KParams& P, int w) {
  return P.ws.scratch + (size_t)w * 2 * P.s.n_up * P.s.det.nao;
}

template <class R, class Tab, class Acc = R>
__global__ void __launch_bounds__(LrdmcShape<R, Acc>::threads, LrdmcShape<R, Acc>::min_ctas) k_lrdmc(KParams P, int K, const double* __restrict__ draw, double alat, double E_scf, double* wgt,
                        double* eL, double* vdiag, TauArgs ta, int emode) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int w = blockIdx.x;
  if (emode == kEnergyGate && !(*energy_bound(P, w) > kFastEnergyCancel)) return;   // uniform over the CTA
  const Sys s = stage_tables(P.s, P.tl, smem);
  Work<Tab> k = make_work<Tab>(s, P.wl, smem, P.ws, w);
  float* gd = (P.dcache_global && sizeof(R) == sizeof(float)) ? P.ws.dcache + (size_t)w * (dcache_floats_dev(s)) : nullptr;
  Terms t = make_terms(P.ml, smem, gd, s);
  load_walker(k, P.ws, w);
  const int N = k.N;
  const bool tmode = ta.tau_left != nullptr;    // GFMC_t: project until the walker's time is spent
  const int dstride = tmode ? 5 : 4, uidx = tmode ? 4 : 3;
  double tleft = tmode ? ta.tau_left[w] : 0.0;
  int done = 0;
  const int nsteps = (tmode && !(tleft > 0.0)) ? 0 : (K > 0 ? K : 1);
  double wl = K > 0 ? wgt[w] : 1.0;
  dcache_fill(k, t);
  for (int step = 0; step < nsteps; ++step) {
    const double* d = draw + ((size_t)w * (K > 0 ? K : 1) + step) * dstride;
    if (threadIdx.x == 0) rotation(d[0], d[1], d[2], t.R);
    __syncthreads();
    if constexpr (sizeof(R) == sizeof(float)) {
      // float rotation and rotated quadrature directions g_v = R m_v (with 1/|g_v|)
      if (threadIdx.x < 9) {
        t.Rf[threadIdx.x] = (float)t.R[threadIdx.x];
      } else if (threadIdx.x >= 32 && threadIdx.x < 32 + s.nv) {
        const int v = threadIdx.x - 32;
        const double* m = s.mesh_pts + 3 * v;
        const double gx = t.R[0] * m[0] + t.R[1] * m[1] + t.R[2] * m[2];
        const double gy = t.R[3] * m[0] + t.R[4] * m[1] + t.R[5] * m[2];
        const double gz = t.R[6] * m[0] + t.R[7] * m[1] + t.R[8] * m[2];
        float* g = t.Rf + 9 + 4 * v;
        g[0] = (float)gx; g[1] = (float)gy; g[2] = (float)gz;
        g[3] = (float)(1.0 / sqrt(gx * gx + gy * gy + gz * gz));
      }
      __syncthreads();
    }
    electron_terms<Tab, Acc>(k, t, alat);
    const Cancellation mc = mesh_terms<R, Tab, Acc>(k, t, alat, true);
    if constexpr (AccTraits<Acc>::accurate && sizeof(Tab) == sizeof(float))
      if (K == 0 && k.tlo_up) {
        refine_lattice(k, t, alat);
        if (s.ecp_flag) mesh_terms<double, Tab, double>(k, t, alat, true, t.vm);   // ECP elements of the heavy electrons
      }
    double diag, nondiag;
    lrdmc_sums(s, k.ec, N, k.red, t, alat, &diag, &nondiag);
    if (K == 0) {
      if (AccTraits<Acc>::accurate && emode == kEnergyBound) {
        const double num = block_sum((double)mc.num, k.red);
        const double den = block_sum((double)mc.den, k.red);
        if (threadIdx.x == 0) *energy_bound(P, w) = den > 0.0 ? num / den : 0.0;
      }
      if (threadIdx.x == 0) {
        eL[w] = diag + nondiag;
        vdiag[w] = diag;
      }
      break;
    }
    if (tmode) {
      // jqmc_gfmc.py:995-1004: continuous-time weight and the time left
      const double el = diag + nondiag;
      const double tu = fmin(tleft, log(1.0 - d[3]) / nondiag);
      wl = wl * exp(-tu * el);
      tleft -= tu;
      ++done;
      if (!(tleft > 0.0)) {
        if (threadIdx.x == 0) ta.eL_last[w] = el;
        break;
      }
    } else {
      wl = wl * (1.0 / (diag - E_scf) * (-1.0 * nondiag));
    }
    const int nk = 6 * N, ne = s.ecp_flag ? s.nv * N : 0, np_ = nk + ne;
    int* kchoice = reinterpret_cast<int*>(k.sc + 31);
    if constexpr (sizeof(Tab) == sizeof(float)) {
      // mixed form: warp-parallel inclusive scan of the normalised FN weights
      if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        const int chunk = (np_ + 31) / 32, p0 = lane * chunk, p1 = min(p0 + chunk, np_);
        double part = 0.0;
        for (int p = p0; p < p1; ++p) part += p < nk ? fmin(t.el[p], 0.0) : fmin(t.V[p - nk], 0.0);
        const double sum = warp_sum(part);
        const double inv = 1.0 / sum;
        double incl = part * inv;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const double v = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += v;
        }
        double cdf = incl - part * inv;   // exclusive prefix of this lane's chunk
        const double u = d[uidx];
        int hit = -1;
        for (int p = p0; p < p1; ++p) {
          cdf += (p < nk ? fmin(t.el[p], 0.0) : fmin(t.V[p - nk], 0.0)) * inv;
          if (cdf >= u) { hit = p; break; }
        }
        const unsigned any = __ballot_sync(0xffffffffu, hit >= 0);
        const int first = __shfl_sync(0xffffffffu, hit, any ? __ffs(any) - 1 : 0);
        if (lane == 0) *kchoice = any ? first : np_ - 1;
      }
    } else {
      // plain form: sequential cumsum in the reference's order (thread 0)
      if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int p = 0; p < nk; ++p) sum += fmin(t.el[p], 0.0);
        for (int q = 0; q < ne; ++q) sum += fmin(t.V[q], 0.0);
        const double u = d[uidx];
        double cdf = 0.0;
        int kk = np_ - 1;
        for (int p = 0; p < np_; ++p) {
          const double x = p < nk ? fmin(t.el[p], 0.0) : fmin(t.V[p - nk], 0.0);
          cdf += x / sum;
          if (cdf >= u) { kk = p; break; }
        }
        *kchoice = kk;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const int kk = *kchoice;
      double px, py, pz;
      int e;
      if (kk < nk) {
        e = kk / 6;
        const int sh = kk % 6, ax = sh >> 1;
        const double sg = (sh & 1) ? -alat : alat;
        px = k.r[3 * e] + sg * t.R[ax];
        py = k.r[3 * e + 1] + sg * t.R[3 + ax];
        pz = k.r[3 * e + 2] + sg * t.R[6 + ax];
      } else {
        const int q = kk - nk, v = q % s.nv;
        e = q / s.nv;
        const int atom = t.eatom[e];
        const double* m = s.mesh_pts + 3 * v;
        const double gx = t.R[0] * m[0] + t.R[1] * m[1] + t.R[2] * m[2];
        const double gy = t.R[3] * m[0] + t.R[4] * m[1] + t.R[5] * m[2];
        const double gz = t.R[6] * m[0] + t.R[7] * m[1] + t.R[8] * m[2];
        const double relx = s.atom_pos[3 * atom] - k.r[3 * e], rely = s.atom_pos[3 * atom + 1] - k.r[3 * e + 1],
                     relz = s.atom_pos[3 * atom + 2] - k.r[3 * e + 2];
        const double dist = sqrt(relx * relx + rely * rely + relz * relz);
        px = k.r[3 * e] + relx + dist * gx;
        py = k.r[3 * e + 1] + rely + dist * gy;
        pz = k.r[3 * e + 2] + relz + dist * gz;
      }
      k.sc[0] = e; k.sc[1] = px; k.sc[2] = py; k.sc[3] = pz;
    }
    __syncthreads();
    const int me = (int)k.sc[0];
    const double mx = k.sc[1], my = k.sc[2], mz = k.sc[3];
    __syncthreads();
    const double ratio = sm_move<Tab>(k, me, mx, my, mz);
    if (threadIdx.x == 0 && ratio == 0.0) atomicOr(P.ws.status + w, JQMC_ST_ZERO_RATIO);
    dcache_update(k, t, me);
  }
  if (K > 0) {
    if (threadIdx.x == 0) {
      wgt[w] = wl;
      if (!isfinite(wl)) atomicOr(P.ws.status + w, JQMC_ST_NAN);
      if (tmode) {
        ta.tau_left[w] = tleft;
        ta.nsteps[w] = done;
      }
    }
    store_walker(k, P.ws, w);
  }
}

__global__ void k_branch_comb(int W, const double* __restrict__ wv, double* cum) {
  // cumulative normalised weights, sequential as np.cumsum (one thread)
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    double tot = 0.0;
    for (int j = 0; j < W; ++j) tot += wv[j];
    double c = 0.0;
    for (int j = 0; j < W; ++j) { c += wv[j] / tot; cum[j] = c; }
  }
}

__global__ void k_branch_search(int W, const double* __restrict__ cum, double zeta, int* chosen) {
  const int kq = blockIdx.x * blockDim.x + threadIdx.x;
  if (kq >= W) return;
  const double z = (kq + zeta) / W;
  int lo = 0, hi = W;  // first j with cum[j] >= z
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (cum[mid] < z) lo = mid + 1; else hi = mid;
  }
  chosen[kq] = lo < W ? lo : W - 1;
}

template <class T>
__global__ void k_gather(const T* __restrict__ src, T* __restrict__ dst, long long per, const int* chosen, int W) {
  const long long tot = per * W;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
    const long long w = t / per, o = t % per;
    dst[t] = src[(long long)chosen[w] * per + o];
  }
}

// FP64 FMA throughput probe: 8 independent FMA chains per thread.
__global__ void k_probe_fp64(long long iters, double* out) {
  double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
  double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
  const double m = 0.999999999, c = 1e-12;
  for (long long i = 0; i < iters; ++i) {
    a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
    a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
  }
  const double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.0) out[0] = s;  // keeps the chains live
}

// FP32 FMA throughput probe: 8 independent FMA chains per thread.
__global__ void k_probe_fp32(long long iters, float* out) {
  float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
  float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
  const float m = 0.9999999f, c = 1e-9f;
  for (long long i = 0; i < iters; ++i) {
    a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
    a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
  }
  const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.0f) out[0] = s;  // keeps the chains live
}

// ------------------------------------------------------------------ host side
inline cudaStream_t S(void* p) { return static_cast<cudaStream_t>(p); }

}  // namespace

struct jqmc_system {
  Sys s;
  void* blob;
  // tensor-core lambda-GEMM of the mixed rebuild (jqmc_tc.cu), when A <= 768:
  // operand B = lambda (spin up) and lambda^T (spin down), split and laid out
  // once; operand A and the row exponents in a workspace grown on first use
  int tc_nk = 0, tc_ncol_tiles = 0;
  uint16_t* tc_b = nullptr;     // [spin][col tile][k chunk][slice][64 x 32]
  int* tc_col_exp = nullptr;    // [spin][col tile * 64]
  uint16_t* tc_a = nullptr;     // [row tile][k chunk][slice][128 x 32]
  int* tc_row_exp = nullptr;
  long long tc_rows_cap = 0;    // rows the workspace holds
};

namespace {

WS to_ws(const jqmc_walkers* w) {
  WS x;
  x.r = w->r; x.G = w->G; x.Ginv = w->Ginv; x.Tup = w->Tup; x.Tdn = w->Tdn; x.h3 = w->h3;
  x.dphi = w->dphi; x.dphi3 = w->dphi3; x.ecache = w->ecache; x.dcache = w->dcache;
  x.scratch = w->scratch; x.status = w->status; x.tlo = w->tlo;
  return x;
}

bool walkers_ok(const jqmc_system* sys, const jqmc_walkers* w) {
  if (!sys || !w || w->nwalk <= 0) return false;
  if (w->precision != JQMC_PREC_FP64 && !is_mixed(w->precision)) return false;
  if (!w->r || !w->G || !w->Ginv || !w->Tup || !w->Tdn || !w->status || !w->dphi || !w->ecache) return false;
  if (sys->s.has_j3 && (!w->h3 || !w->dphi3)) return false;
  if (is_mixed(w->precision) && !w->scratch) return false;
  if (is_mixed(w->precision) && dcache_bytes(sys->s) > kDcacheSmemMax && !w->dcache) return false;
  return true;
}

int tab_bytes(const jqmc_walkers* w) { return is_mixed(w->precision) ? 4 : 8; }

KParams make_params(const jqmc_system* sys, const jqmc_walkers* w) {
  KParams P;
  P.s = sys->s;
  P.ws = to_ws(w);
  const bool mixed = is_mixed(w->precision);
  P.tl = table_layout(sys->s, !mixed);
  P.wl = work_layout(sys->s, P.tl.bytes, tab_bytes(w));
  P.dcache_global = mixed && dcache_bytes(sys->s) > kDcacheSmemMax;
  P.ml = terms_layout(sys->s, P.wl.bytes, mixed && !P.dcache_global);
  P.nwalk = w->nwalk;
  return P;
}

// Raise a kernel's dynamic shared-memory limit when a launch needs more than
// was set before on this device (so launches inside a stream capture make no
// attribute calls once the kernels have run at their sizes).
int launch_check(const void* fn, int smem) {
  if (smem > 227 * 1024) return JQMC_E_SMEM;
  static std::mutex mu;
  static std::vector<std::pair<std::pair<const void*, int>, int>> done;   // ((kernel, device), bytes)
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return JQMC_E_CUDA;
  std::lock_guard<std::mutex> lock(mu);
  for (auto& d : done)
    if (d.first.first == fn && d.first.second == dev) {
      if (smem <= d.second) return JQMC_OK;
      if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) return JQMC_E_CUDA;
      d.second = smem;
      return JQMC_OK;
    }
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) return JQMC_E_CUDA;
  done.push_back({{fn, dev}, smem});
  return JQMC_OK;
}

// Square of the radius beyond which sum_q |c_q| max(r, 1)^l exp(-Z_q r^2), a
// bound on every AO of shell k (|solid harmonic| <= r^l with the prefactor in
// c_q; Cartesian monomials likewise), stays below e^-C.  The bound decreases
// for r past its last crossing, found on a 0.05-bohr grid out to 100 bohr; the
// radius is rounded up by one grid step.
double shell_reach2(const jqmc_basis_desc& b, int k, double C) {
  const int32_t* sh = b.shells + 8 * (size_t)k;
  const int l = sh[1], np = sh[2], p0 = sh[3];
  const double lim = std::exp(-C);
  double last = 0.0;
  for (int i = 0; i <= 2000; ++i) {
    const double r = 0.05 * i;
    double f = 0.0;
    for (int q = 0; q < np; ++q) f += std::fabs(b.prims[2 * (p0 + q) + 1]) * std::exp(-b.prims[2 * (p0 + q)] * r * r);
    f *= std::pow(r > 1.0 ? r : 1.0, l);
    if (f >= lim) last = r;
  }
  const double R = last + 0.05;
  return R * R;
}

int launch_lrdmc(const jqmc_system* sys, const jqmc_walkers* w, int K, const double* d_draw, double alat, double E_scf,
                 double* d_w, double* d_eL, double* d_vd, void* stream, TauArgs ta = TauArgs{nullptr, nullptr, nullptr}) {
  KParams P = make_params(sys, w);
  const int smem = terms_smem(P.ml, LrdmcShape<double, double>::threads);   // 4-warp kernels
  if (is_mixed(w->precision)) {
    // projections: float arithmetic on the float tables.  The local energy of a
    // block (K == 0): float values with compensated float-float sums, then FP64
    // arithmetic for the walkers whose cancellation factor exceeds
    // JQMC_FAST_ENERGY_CANCEL (JQMC_PREC_MIXED), or the compensated energy alone
    // (JQMC_PREC_MIXED_FASTE)
    if (K > 0) {
      auto fn = k_lrdmc<float, float, float>;
      const int smem_p = terms_smem(P.ml, 0);   // float mesh ratios only
      int rc = launch_check((const void*)fn, smem_p);
      if (rc) return rc;
      fn<<<w->nwalk, LrdmcShape<float, float>::threads, smem_p, S(stream)>>>(P, K, d_draw, alat, E_scf, d_w, d_eL, d_vd, ta, kEnergyPlain);
    } else {
      const bool gate = w->precision == JQMC_PREC_MIXED;
      auto fn = k_lrdmc<float, float, F2>;
      const int smem_e = terms_smem(P.ml, LrdmcShape<float, F2>::threads);
      int rc = launch_check((const void*)fn, smem_e);
      if (rc) return rc;
      fn<<<w->nwalk, LrdmcShape<float, F2>::threads, smem_e, S(stream)>>>(P, K, d_draw, alat, E_scf, d_w, d_eL, d_vd, ta,
                                                                         gate ? kEnergyBound : kEnergyPlain);
      if (gate) {
        auto fd = k_lrdmc<double, float, double>;
        rc = launch_check((const void*)fd, smem);
        if (rc) return rc;
        fd<<<w->nwalk, LrdmcShape<double, double>::threads, smem, S(stream)>>>(P, K, d_draw, alat, E_scf, d_w, d_eL, d_vd, ta, kEnergyGate);
      }
    }
  } else {
    auto fn = k_lrdmc<double, double>;
    int rc = launch_check((const void*)fn, smem);
    if (rc) return rc;
    fn<<<w->nwalk, LrdmcShape<double, double>::threads, smem, S(stream)>>>(P, K, d_draw, alat, E_scf, d_w, d_eL, d_vd, ta,
                                                                           kEnergyPlain);
  }
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

}  // namespace

extern "C" {

int jqmc_system_create(const jqmc_system_desc* d, jqmc_system** out) {
  if (!d || !out) return JQMC_E_ARG;
  *out = nullptr;
  const int M = d->natom, A = d->det.nao;
  if (M <= 0 || M > JQMC_MAX_ATOM || d->n_up <= 0 || d->n_up > JQMC_MAX_NUP) return JQMC_E_LIMIT;
  if (d->n_up != d->n_dn) return JQMC_E_ARG;  // the walker kernels treat closed shells
  if (d->n_up + d->n_dn > JQMC_MAX_ELEC || A <= 0 || A > JQMC_MAX_AO) return JQMC_E_LIMIT;
  if (d->n_up > A) return JQMC_E_ARG;          // G would be singular
  if (!d->atom_pos || !d->atom_zeff || !d->lambda || !d->det.shells || !d->det.prims) return JQMC_E_ARG;
  const int A3 = d->has_j3 ? d->j3.nao : 0;
  if (d->has_j3 && (A3 <= 0 || A3 > JQMC_MAX_AO || !d->j3.shells || !d->j3.prims || !d->j3_matrix)) return JQMC_E_ARG;
  if (d->has_j1 && !d->j1_zeff) return JQMC_E_ARG;
  if (d->ecp_flag && (!d->ecp_maxl1 || !d->ecp_chan || !d->ecp_terms || !d->mesh_points || !d->mesh_weights)) return JQMC_E_ARG;
  if (d->ecp_flag && !(d->nv == 4 || d->nv == 6 || d->nv == 12 || d->nv == 18)) return JQMC_E_ARG;
  if (d->nonlocal_move != JQMC_NONLOCAL_TMOVE && d->nonlocal_move != JQMC_NONLOCAL_DLTMOVE) return JQMC_E_ARG;
  auto check_basis = [M](const jqmc_basis_desc& b) {
    int prev_atom = -1;
    for (int s = 0; s < b.nshell; ++s) {
      const int* sh = b.shells + 8 * s;
      if (sh[0] < 0 || sh[0] >= M || sh[0] < prev_atom) return false;  // shells grouped by nucleus
      prev_atom = sh[0];
      if (sh[1] < 0 || sh[1] > JQMC_LMAX || sh[2] <= 0 || sh[3] < 0 || sh[3] + sh[2] > b.nprim) return false;
      if (sh[7] != 0 && sh[7] != 1) return false;
      if (sh[7] == 1) {   // Cartesian: one AO, component index below (l+1)(l+2)/2
        if (sh[5] != 1 || sh[6] < 0 || sh[6] >= (sh[1] + 1) * (sh[1] + 2) / 2 || sh[4] < 0 || sh[4] >= b.nao) return false;
      } else if (sh[5] <= 0 || sh[6] < -sh[1] || sh[6] + sh[5] - 1 > sh[1] || sh[4] < 0 || sh[4] + sh[5] > b.nao) {
        return false;
      }
    }
    return true;
  };
  if (!check_basis(d->det) || (d->has_j3 && !check_basis(d->j3))) return JQMC_E_ARG;
  if (d->ecp_flag)
    for (int a = 0; a < M; ++a) {
      if (d->ecp_maxl1[a] < 0 || d->ecp_maxl1[a] >= kSlots) return JQMC_E_ARG;
      for (int l = 0; l < kSlots; ++l) {
        const int* ch = d->ecp_chan + (a * kSlots + l) * 2;
        if (ch[1] < 0 || ch[0] < 0 || ch[0] + ch[1] > d->ecp_nterm) return JQMC_E_ARG;
      }
    }

  // one device blob for every table
  std::vector<unsigned char> host;
  auto put = [&host](const void* src, size_t bytes) -> size_t {
    const size_t off = (host.size() + 255) & ~size_t(255);
    host.resize(off + (bytes ? bytes : 8));
    if (bytes) memcpy(host.data() + off, src, bytes);
    return off;
  };
  std::vector<double> lamT((size_t)A * A);
  std::vector<float> lamf((size_t)A * A), lamTf((size_t)A * A), laml((size_t)A * A), lamTl((size_t)A * A);
  for (int a = 0; a < A; ++a)
    for (int b = 0; b < A; ++b) {
      const double v = d->lambda[(size_t)a * A + b];
      lamT[(size_t)b * A + a] = v;
      lamf[(size_t)a * A + b] = (float)v;
      lamTf[(size_t)b * A + a] = (float)v;
      laml[(size_t)a * A + b] = (float)(v - (double)(float)v);
      lamTl[(size_t)b * A + a] = (float)(v - (double)(float)v);
    }
  std::vector<double> j3m, j3mT, j3v;
  std::vector<float> j3mf, j3mTf, j3k4;
  if (d->has_j3) {
    j3m.resize((size_t)A3 * A3);
    j3mT.resize((size_t)A3 * A3);
    j3mf.resize((size_t)A3 * A3);
    j3mTf.resize((size_t)A3 * A3);
    j3k4.resize((size_t)A3 * A3 * 4);
    j3v.resize(A3);
    for (int a = 0; a < A3; ++a) {
      for (int b = 0; b < A3; ++b) {
        const double v = d->j3_matrix[(size_t)a * (A3 + 1) + b];
        j3m[(size_t)a * A3 + b] = v;
        j3mT[(size_t)b * A3 + a] = v;
        j3mf[(size_t)a * A3 + b] = (float)v;
        j3mTf[(size_t)b * A3 + a] = (float)v;
      }
      j3v[a] = d->j3_matrix[(size_t)a * (A3 + 1) + A3];
    }
    for (int cp = 0; cp < A3; ++cp)
      for (int c = 0; c < A3; ++c) {
        const double x = d->j3_matrix[(size_t)cp * (A3 + 1) + c], y = d->j3_matrix[(size_t)c * (A3 + 1) + cp];
        float* q = &j3k4[((size_t)cp * A3 + c) * 4];
        q[0] = (float)x; q[1] = (float)(x - (double)q[0]);
        q[2] = (float)y; q[3] = (float)(y - (double)q[2]);
      }
  }
  auto to_float = [](const double* p, size_t n) { std::vector<float> v(n); for (size_t i = 0; i < n; ++i) v[i] = (float)p[i]; return v; };
  std::vector<float> dprf = to_float(d->det.prims, (size_t)d->det.nprim * 2);
  std::vector<float> jprf = d->has_j3 ? to_float(d->j3.prims, (size_t)d->j3.nprim * 2) : std::vector<float>();
  std::vector<double> zero(2 * M, 0.0);
  std::vector<int> zeroi(M * kSlots * 2 + M, 0);
  std::vector<double> j1cA(2 * M, 0.0);
  if (d->has_j1)
    for (int a = 0; a < M; ++a) {
      j1cA[2 * a] = pow(2.0 * d->j1_zeff[a], 0.25);
      j1cA[2 * a + 1] = pow(2.0 * d->j1_zeff[a], 0.75);
    }
  const size_t o_apos = put(d->atom_pos, (size_t)M * 24);
  const size_t o_az = put(d->atom_zeff, (size_t)M * 8);
  // Shell rows are copied at the device stride kSh with their 8th int set to a permutation of the shells
  // sorted by (l, nprim): the warp-cooperative mesh evaluation walks the shells
  // in that order, so the 32 lanes of an iteration take the same code path.
  auto with_order = [](const jqmc_basis_desc& b) {
    std::vector<int32_t> rows(b.shells, b.shells + (size_t)b.nshell * 8);
    std::vector<int32_t> ord(b.nshell);
    for (int k = 0; k < b.nshell; ++k) ord[k] = k;
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) {
      const int lx = rows[8 * x + 1], ly = rows[8 * y + 1];
      return lx != ly ? lx < ly : rows[8 * x + 2] < rows[8 * y + 2];
    });
    std::vector<int32_t> dev((size_t)b.nshell * kSh, 0);   // padded to the device stride
    for (int k = 0; k < b.nshell; ++k) {
      for (int f = 0; f < 8; ++f) dev[(size_t)kSh * k + f] = rows[8 * k + f];
      if (rows[8 * k + 7] == 1) dev[(size_t)kSh * k + 6] += kCartBase;   // the Cartesian kind moves to field 6
      dev[(size_t)kSh * k + 7] = ord[k];
      const float r2 = (float)shell_reach2(b, k, kReach);
      std::memcpy(&dev[(size_t)kSh * k + kShReach], &r2, 4);
    }
    return dev;
  };
  const std::vector<int32_t> dsh_rows = with_order(d->det);
  const size_t o_dsh = put(dsh_rows.data(), dsh_rows.size() * 4);
  const size_t o_dpr = put(d->det.prims, (size_t)d->det.nprim * 16);
  const size_t o_dprf = put(dprf.data(), dprf.size() * 4);
  const size_t o_lam = put(d->lambda, (size_t)A * A * 8);
  const size_t o_lamT = put(lamT.data(), (size_t)A * A * 8);
  const size_t o_lamf = put(lamf.data(), (size_t)A * A * 4);
  const size_t o_lamTf = put(lamTf.data(), (size_t)A * A * 4);
  const size_t o_laml = put(laml.data(), (size_t)A * A * 4);
  const size_t o_lamTl = put(lamTl.data(), (size_t)A * A * 4);
  const size_t o_j1z = put(j1cA.data(), (size_t)M * 16);
  size_t o_jsh = 0, o_jpr = 0, o_jprf = 0, o_j3m = 0, o_j3mT = 0, o_j3v = 0, o_j3mf = 0, o_j3mTf = 0, o_j3k4 = 0;
  if (d->has_j3) {
    const std::vector<int32_t> jsh_rows = with_order(d->j3);
    o_jsh = put(jsh_rows.data(), jsh_rows.size() * 4);
    o_jpr = put(d->j3.prims, (size_t)d->j3.nprim * 16);
    o_jprf = put(jprf.data(), jprf.size() * 4);
    o_j3m = put(j3m.data(), j3m.size() * 8);
    o_j3mT = put(j3mT.data(), j3mT.size() * 8);
    o_j3v = put(j3v.data(), j3v.size() * 8);
    o_j3mf = put(j3mf.data(), j3mf.size() * 4);
    o_j3mTf = put(j3mTf.data(), j3mTf.size() * 4);
    o_j3k4 = put(j3k4.data(), j3k4.size() * 4);
  }
  const size_t o_maxl1 = put(d->ecp_flag ? d->ecp_maxl1 : zeroi.data(), (size_t)M * 4);
  const size_t o_chan = put(d->ecp_flag ? d->ecp_chan : zeroi.data(), (size_t)M * kSlots * 8);
  const size_t o_terms = put(d->ecp_flag ? d->ecp_terms : zero.data(), (size_t)(d->ecp_flag ? d->ecp_nterm : 1) * 24);
  const int nv = d->ecp_flag ? d->nv : 0;
  const size_t o_mp = put(d->ecp_flag ? d->mesh_points : zero.data(), (size_t)(nv > 0 ? nv : 1) * 24);
  const size_t o_mw = put(d->ecp_flag ? d->mesh_weights : zero.data(), (size_t)(nv > 0 ? nv : 1) * 8);

  void* blob = nullptr;
  if (cudaMalloc(&blob, host.size()) != cudaSuccess) return JQMC_E_CUDA;
  if (cudaMemcpy(blob, host.data(), host.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(blob);
    return JQMC_E_CUDA;
  }
  auto dp = [blob](size_t off) { return reinterpret_cast<const double*>(static_cast<unsigned char*>(blob) + off); };
  auto fp = [blob](size_t off) { return reinterpret_cast<const float*>(static_cast<unsigned char*>(blob) + off); };
  auto ip = [blob](size_t off) { return reinterpret_cast<const int*>(static_cast<unsigned char*>(blob) + off); };
  jqmc_system* sys = new jqmc_system();
  Sys& s = sys->s;
  s.natom = M; s.n_up = d->n_up; s.n_dn = d->n_dn; s.N = d->n_up + d->n_dn;
  s.atom_pos = dp(o_apos); s.atom_zeff = dp(o_az);
  s.det.nshell = d->det.nshell; s.det.nao = A; s.det.nprim = d->det.nprim;
  s.det.shells = ip(o_dsh); s.det.prims = dp(o_dpr); s.det.primsf = fp(o_dprf);
  s.lam = dp(o_lam); s.lamT = dp(o_lamT); s.lamf = fp(o_lamf); s.lamTf = fp(o_lamTf);
  s.laml = fp(o_laml); s.lamTl = fp(o_lamTl);
  s.has_j1 = d->has_j1; s.j1_type = d->j1_type; s.j1_param = d->j1_param; s.j1_cA = dp(o_j1z);
  s.has_j2 = d->has_j2; s.j2_type = d->j2_type; s.j2_param = d->j2_param;
  s.has_j3 = d->has_j3;
  if (d->has_j3) {
    s.j3.nshell = d->j3.nshell; s.j3.nao = A3; s.j3.nprim = d->j3.nprim;
    s.j3.shells = ip(o_jsh); s.j3.prims = dp(o_jpr); s.j3.primsf = fp(o_jprf);
    s.j3mat = dp(o_j3m); s.j3matT = dp(o_j3mT); s.j3vec = dp(o_j3v); s.j3matf = fp(o_j3mf); s.j3matTf = fp(o_j3mTf);
    s.j3k4 = reinterpret_cast<const float4*>(fp(o_j3k4));
  } else {
    s.j3.nshell = 0; s.j3.nao = 0; s.j3.nprim = 0; s.j3.shells = nullptr; s.j3.prims = nullptr; s.j3.primsf = nullptr;
    s.j3mat = s.j3matT = s.j3vec = nullptr;
    s.j3matf = s.j3matTf = nullptr;
    s.j3k4 = nullptr;
  }
  s.ecp_flag = d->ecp_flag;
  s.ecp_maxl1 = ip(o_maxl1); s.ecp_chan = ip(o_chan);
  s.ecp_nterm = d->ecp_flag ? d->ecp_nterm : 0; s.ecp_terms = dp(o_terms);
  s.nv = nv; s.mesh_pts = dp(o_mp); s.mesh_w = dp(o_mw);
  s.ion_ion = d->ion_ion;
  s.dlt = d->nonlocal_move == JQMC_NONLOCAL_DLTMOVE;
  sys->blob = blob;
  if (A <= jqmc_tc::kMaxK) {
    // operand B of the tensor-core lambda-GEMM: column b of L = lambda (spin up:
    // M_up = Phi_up lambda) or lambda^T (spin down: M_dn rows = lambda phi_dn),
    // scaled by 2^-e_b and split into six 8-bit slices (bf16), in the tensor
    // cores' layout [spin][col tile][k chunk][slice][64 x 32 canonical block]
    using namespace jqmc_tc;
    const int nk = (A + kKC - 1) / kKC, nct = (A + kBN - 1) / kBN;
    const size_t per_spin = (size_t)nct * nk * kBStage / 2;   // bf16 elements
    std::vector<uint16_t> hb(2 * per_spin, 0);
    std::vector<int> hexp((size_t)2 * nct * kBN, 0);
    for (int spin = 0; spin < 2; ++spin)
      for (int b = 0; b < A; ++b) {
        auto L = [&](int a) { return spin == 0 ? d->lambda[(size_t)a * A + b] : d->lambda[(size_t)b * A + a]; };
        double m = 0.0;
        for (int a = 0; a < A; ++a) m = std::max(m, fabs(L(a)));
        int e = 0;
        if (m > 0.0) frexp(m, &e);
        hexp[(size_t)spin * nct * kBN + b] = e;
        const int ct = b / kBN, rb = b % kBN;
        for (int a = 0; a < A; ++a) {
          float q[kSlices];
          split8(ldexp(L(a), -e), q);
          const int c = a / kKC, kk = a % kKC;
          for (int sl = 0; sl < kSlices; ++sl) {
            uint32_t bits;
            memcpy(&bits, &q[sl], 4);   // 8 significant bits at most: the high half is its exact bf16
            const size_t off = ((size_t)ct * nk + c) * kBStage + (size_t)sl * kBSliceBytes + canon_offset(rb, kk);
            hb[spin * per_spin + off / 2] = (uint16_t)(bits >> 16);
          }
        }
      }
    if (cudaMalloc(&sys->tc_b, hb.size() * 2) != cudaSuccess ||
        cudaMalloc(&sys->tc_col_exp, hexp.size() * sizeof(int)) != cudaSuccess ||
        cudaMemcpy(sys->tc_b, hb.data(), hb.size() * 2, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(sys->tc_col_exp, hexp.data(), hexp.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
      if (sys->tc_b) cudaFree(sys->tc_b);
      if (sys->tc_col_exp) cudaFree(sys->tc_col_exp);
      cudaFree(blob);
      delete sys;
      return JQMC_E_CUDA;
    }
    sys->tc_nk = nk;
    sys->tc_ncol_tiles = nct;
  }
  *out = sys;
  return JQMC_OK;
}

int32_t jqmc_tensor_core_rebuild(const jqmc_system* sys) { return sys ? (sys->tc_b ? 1 : 0) : JQMC_E_ARG; }

int jqmc_system_destroy(jqmc_system* sys) {
  if (!sys) return JQMC_E_ARG;
  cudaDeviceSynchronize();
  if (sys->blob) cudaFree(sys->blob);
  if (sys->tc_b) cudaFree(sys->tc_b);
  if (sys->tc_col_exp) cudaFree(sys->tc_col_exp);
  if (sys->tc_a) cudaFree(sys->tc_a);
  if (sys->tc_row_exp) cudaFree(sys->tc_row_exp);
  delete sys;
  return JQMC_OK;
}

int64_t jqmc_walker_bytes(const jqmc_system* sys, int32_t precision) {
  if (!sys || (precision != JQMC_PREC_FP64 && !is_mixed(precision))) return JQMC_E_ARG;
  const Sys& s = sys->s;
  const int64_t n = s.n_up, N = s.N, A = s.det.nao, A3 = s.has_j3 ? s.j3.nao : 0;
  const int64_t tb = is_mixed(precision) ? 4 : 8;
  return 8 * N * 3 + 8 * (N + 1) * kEC + tb * (2 * n * n + 2 * n * A + N * A3 + N * 4 * A + N * 5 * A3) + 4 +
         (is_mixed(precision) ? 8 * 2 * n * A : 0);
}

int jqmc_ao_vgl(const jqmc_system* sys, int32_t basis, const double* d_r, int64_t npts, double* d_out, void* stream) {
  if (!sys || !d_r || !d_out || npts < 0 || (basis != 0 && basis != 1)) return JQMC_E_ARG;
  if (basis == 1 && !sys->s.has_j3) return JQMC_E_ARG;
  if (npts == 0) return JQMC_OK;
  const int bs = 128;
  k_ao_vgl<<<(unsigned)((npts + bs - 1) / bs), bs, 0, S(stream)>>>(sys->s, basis, d_r, npts, d_out);
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

// shared-memory layout of the init / rebuild kernel above the work layout; returns the bytes
// The rebuild's shared memory: the positions, the reduction buffer and the
// pivot slot, then G, [G | I] and the vectors -- no staged tables and none of
// the energy kernels' work buffers, so that three CTAs fit on an SM.
static InitLayout init_layout(const Sys& s, const KParams&) {
  const int n = s.n_up, A3 = s.has_j3 ? s.j3.nao : 1;
  InitLayout L;
  int o = 0;
  L.r = o; o = align16(o + s.N * 3 * 8);
  L.red = o; o = align16(o + kRed * 8);
  L.sc = o; o = align16(o + 32 * 8);
  L.Gd = o; o = align16(o + n * n * 8);                  // G (double)
  L.aug = o; o = align16(o + n * 2 * n * 8);             // [G | I]
  const int vec_len = (s.det.nao + n > 4 * A3) ? s.det.nao + n : 4 * A3;
  L.vec = o; o = align16(o + vec_len * 8);
  L.bytes = o;
  return L;
}

// M_up / M_dn of the mixed rebuild on the tensor cores (k_ao_slices +
// jqmc_tc::ozaki_gemm) into the walkers' scratch, in chunks of at most 65536
// electron rows per spin (the operand workspace, about 0.6 GB for A = 736, is
// allocated on first use and kept with the system).  Returns kTcUnavailable
// when the workspace would have to grow inside a stream capture; the caller
// then uses the CUDA-core kernel.
constexpr int kTcUnavailable = 1;
static int tc_rebuild_m(const jqmc_system* csys, const jqmc_walkers* w, const KParams& P, void* stream) {
  using namespace jqmc_tc;
  jqmc_system* sys = const_cast<jqmc_system*>(csys);   // the workspace is a cache of the system
  const Sys& s = sys->s;
  const int n = s.n_up, A = s.det.nao, nk = sys->tc_nk, nct = sys->tc_ncol_tiles;
  const long long rows_total = (long long)w->nwalk * n;
  const long long want = ((std::min(rows_total, 65536ll) + kBM - 1) / kBM) * kBM;
  if (sys->tc_rows_cap < want) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(S(stream), &cs) != cudaSuccess) return JQMC_E_CUDA;
    if (cs != cudaStreamCaptureStatusNone) return kTcUnavailable;
    if (cudaStreamSynchronize(S(stream)) != cudaSuccess) return JQMC_E_CUDA;   // the old workspace may be in use
    if (sys->tc_a) cudaFree(sys->tc_a);
    if (sys->tc_row_exp) cudaFree(sys->tc_row_exp);
    sys->tc_a = nullptr;
    sys->tc_row_exp = nullptr;
    sys->tc_rows_cap = 0;
    if (cudaMalloc(&sys->tc_a, (size_t)(want / kBM) * nk * kAStage) != cudaSuccess ||
        cudaMalloc(&sys->tc_row_exp, (size_t)want * sizeof(int)) != cudaSuccess)
      return JQMC_E_CUDA;
    sys->tc_rows_cap = want;
  }
  const int smem_a = 8 * nk * kKC * 8;
  int rc = launch_check((const void*)k_ao_slices, smem_a);
  if (rc) return rc;
  const size_t b_spin = (size_t)nct * nk * kBStage / 2;
  for (int spin = 0; spin < 2; ++spin)
    for (long long r0 = 0; r0 < rows_total; r0 += sys->tc_rows_cap) {
      const long long rows = std::min(sys->tc_rows_cap, rows_total - r0);
      const int tiles = (int)((rows + kBM - 1) / kBM);
      // the down spin also leaves phi_dn as float pairs over T_up (hi) and T_dn (lo)
      k_ao_slices<<<tiles * (kBM / 8), 128, smem_a, S(stream)>>>(
          P, spin, r0, rows_total, nk, reinterpret_cast<uint8_t*>(sys->tc_a), sys->tc_row_exp,
          spin == 1 ? static_cast<float*>(w->Tup) : nullptr, spin == 1 ? static_cast<float*>(w->Tdn) : nullptr);
      rc = ozaki_gemm(sys->tc_a, sys->tc_b + spin * b_spin, sys->tc_row_exp, sys->tc_col_exp + (size_t)spin * nct * kBN, nk,
                      nct, tiles, r0, rows_total, n, A, spin == 0 ? 1 : 0, reinterpret_cast<float2*>(w->scratch), w->status,
                      JQMC_ST_NAN, S(stream));
      if (rc) return JQMC_E_CUDA;
    }
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

static int launch_walker_init(const jqmc_system* sys, const jqmc_walkers* w, void* stream, int mode) {
  if (!walkers_ok(sys, w)) return JQMC_E_ARG;
  KParams P = make_params(sys, w);
  const Sys& s = sys->s;
  const int n = s.n_up;
  const InitLayout IL = init_layout(s, P);
  const int smem = IL.bytes;
  if (is_mixed(w->precision)) {
    // M_up, M_dn into the scratch: by the split-bf16 tensor-core GEMM when the
    // system has its operand (A <= 768), else by the float-float CUDA-core
    // kernel; then the rest in FP64
    int rc = sys->tc_b ? tc_rebuild_m(sys, w, P, stream) : kTcUnavailable;
    if (rc < 0) return rc;
    if (rc == kTcUnavailable) {
      const int rows = s.det.nao <= 2048 ? 8 : 4;
      const int smem_m = rows * s.det.nao * 8;
      const void* fm = rows == 8 ? (const void*)k_rebuild_m<8> : (const void*)k_rebuild_m<4>;
      rc = launch_check(fm, smem_m);
      if (rc) return rc;
      const dim3 grid_m(w->nwalk, 2 * ((n + rows - 1) / rows));
      if (rows == 8) k_rebuild_m<8><<<grid_m, 128, smem_m, S(stream)>>>(P);
      else k_rebuild_m<4><<<grid_m, 128, smem_m, S(stream)>>>(P);
    }
    const int phi = rc == kTcUnavailable ? 0 : kInitPhiReady;
    rc = launch_check((const void*)k_walker_init<float>, smem);
    if (rc) return rc;
    k_walker_init<float><<<w->nwalk, 128, smem, S(stream)>>>(P, IL, mode | kInitMReady | phi);
  } else {
    int rc = launch_check((const void*)k_walker_init<double>, smem);
    if (rc) return rc;
    k_walker_init<double><<<w->nwalk, 128, smem, S(stream)>>>(P, IL, mode);
  }
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

int jqmc_walker_init(const jqmc_system* sys, const jqmc_walkers* w, void* stream) {
  return launch_walker_init(sys, w, stream, 0);
}

int jqmc_lu_rebuild_refine(const jqmc_system* sys, const jqmc_walkers* w, void* stream) {
  return launch_walker_init(sys, w, stream, kInitTablesOnly | kInitRefine);
}

int jqmc_log_psi(const jqmc_system* sys, const jqmc_walkers* w, double* d_logdet, double* d_sign, double* d_jastrow,
                 void* stream) {
  if (!walkers_ok(sys, w) || !d_logdet || !d_sign || !d_jastrow) return JQMC_E_ARG;
  if (w->precision != JQMC_PREC_FP64) return JQMC_E_ARG;
  KParams P = make_params(sys, w);
  const int off_aug = P.wl.bytes;
  const int smem = align16(off_aug + sys->s.n_up * sys->s.n_up * 8);
  int rc = launch_check((const void*)k_log_psi, smem);
  if (rc) return rc;
  k_log_psi<<<w->nwalk, 128, smem, S(stream)>>>(P, off_aug, d_logdet, d_sign, d_jastrow);
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

int jqmc_kinetic_mesh(const jqmc_system* sys, const jqmc_walkers* w, const double* d_angles, double alat, double* d_el,
                      void* stream) {
  if (!walkers_ok(sys, w) || w->precision != JQMC_PREC_FP64 || !d_angles || !d_el || !(alat > 0.0)) return JQMC_E_ARG;
  KParams P = make_params(sys, w);
  const int smem = terms_smem(P.ml, 128);
  int rc = launch_check((const void*)k_kinetic_mesh, smem);
  if (rc) return rc;
  k_kinetic_mesh<<<w->nwalk, 128, smem, S(stream)>>>(P, d_angles, alat, d_el);
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

int jqmc_electron_terms(const jqmc_system* sys, const jqmc_walkers* w, double* d_out, void* stream) {
  if (!walkers_ok(sys, w) || w->precision != JQMC_PREC_FP64 || !d_out) return JQMC_E_ARG;
  KParams P = make_params(sys, w);
  const int smem = P.wl.bytes;
  int rc = launch_check((const void*)k_electron_terms, smem);
  if (rc) return rc;
  k_electron_terms<<<w->nwalk, 128, smem, S(stream)>>>(P, d_out);
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

int jqmc_dlnpsi_dparam(const jqmc_system* sys, const jqmc_walkers* w, double* d_j1, double* d_j2, double* d_j3,
                       double* d_lambda, double* d_work, void* stream) {
  if (!walkers_ok(sys, w) || w->precision != JQMC_PREC_FP64) return JQMC_E_ARG;
  if (d_lambda && !d_work) return JQMC_E_ARG;
  const Sys& s = sys->s;
  KParams P = make_params(sys, w);
  const int A3 = s.has_j3 ? s.j3.nao : 1;
  const int off_red = align16(s.N * 3 * 8);
  const int off_su = align16(off_red + 33 * 8);
  const int off_sd = align16(off_su + A3 * 8);
  const int off_phi3 = align16(off_sd + A3 * 8);
  const int smem = align16(off_phi3 + (s.has_j3 ? s.N * A3 * 8 : 8));
  int rc = launch_check((const void*)k_dlnpsi_dparam, smem);
  if (rc) return rc;
  k_dlnpsi_dparam<<<w->nwalk, 128, smem, S(stream)>>>(P, off_red, off_su, off_sd, off_phi3, d_j1, d_j2,
                                                      s.has_j3 ? d_j3 : nullptr, d_lambda, d_work);
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

int jqmc_dlnpsi_dR(const jqmc_system* sys, const jqmc_walkers* w, double* d_out, void* stream) {
  if (!walkers_ok(sys, w) || w->precision != JQMC_PREC_FP64 || !d_out) return JQMC_E_ARG;
  KParams P = make_params(sys, w);
  const int off_acc = P.wl.bytes;
  const int smem = align16(off_acc + sys->s.natom * 3 * 8);
  int rc = launch_check((const void*)k_dlnpsi_dR, smem);
  if (rc) return rc;
  k_dlnpsi_dR<<<w->nwalk, 128, smem, S(stream)>>>(P, off_acc, d_out);
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

int jqmc_vmc_sweep(const jqmc_system* sys, const jqmc_walkers* w, int32_t K, const int32_t* d_idraw,
                   const double* d_fdraw, double Dt, double eps_AS, int32_t* d_accept, void* stream) {
  if (!walkers_ok(sys, w) || K < 0 || !d_idraw || !d_fdraw || !d_accept) return JQMC_E_ARG;
  if (w->precision != JQMC_PREC_FP64) return JQMC_E_ARG;
  if (K == 0) return JQMC_OK;
  KParams P = make_params(sys, w);
  const int off_cand = P.wl.bytes;
  const int smem = align16(off_cand + 2 * sys->s.n_up * sys->s.n_up * 8);
  int rc = launch_check((const void*)k_vmc_sweep, smem);
  if (rc) return rc;
  k_vmc_sweep<<<w->nwalk, 64, smem, S(stream)>>>(P, K, d_idraw, d_fdraw, Dt, eps_AS, d_accept, off_cand);
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

int jqmc_vmc_measure(const jqmc_system* sys, const jqmc_walkers* w, const double* d_angles, double eps_AS,
                     double* d_eL, double* d_wL, void* stream) {
  if (!walkers_ok(sys, w) || !d_angles || !d_eL || !d_wL) return JQMC_E_ARG;
  if (w->precision != JQMC_PREC_FP64) return JQMC_E_ARG;
  KParams P = make_params(sys, w);
  const int smem = terms_smem(P.ml, 128);
  int rc = launch_check((const void*)k_vmc_measure, smem);
  if (rc) return rc;
  k_vmc_measure<<<w->nwalk, 128, smem, S(stream)>>>(P, d_angles, eps_AS, d_eL, d_wL);
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

int jqmc_lrdmc_project(const jqmc_system* sys, const jqmc_walkers* w, int32_t K, const double* d_draw, double alat,
                       double E_scf, double* d_w, void* stream) {
  if (!walkers_ok(sys, w) || K < 0 || !d_draw || !d_w || !(alat > 0.0)) return JQMC_E_ARG;
  if (K == 0) return JQMC_OK;
  return launch_lrdmc(sys, w, K, d_draw, alat, E_scf, d_w, nullptr, nullptr, stream);
}

int jqmc_lrdmc_energy(const jqmc_system* sys, const jqmc_walkers* w, const double* d_draw, double alat, double* d_eL,
                      double* d_vdiag, void* stream) {
  if (!walkers_ok(sys, w) || !d_draw || !d_eL || !d_vdiag || !(alat > 0.0)) return JQMC_E_ARG;
  return launch_lrdmc(sys, w, 0, d_draw, alat, 0.0, nullptr, d_eL, d_vdiag, stream);
}

int jqmc_lrdmc_project_t(const jqmc_system* sys, const jqmc_walkers* w, int32_t K, const double* d_draw, double alat,
                         double* d_w, double* d_tau_left, int32_t* d_nsteps, double* d_eL, void* stream) {
  if (!walkers_ok(sys, w) || K <= 0 || !d_draw || !d_w || !d_tau_left || !d_nsteps || !d_eL || !(alat > 0.0))
    return JQMC_E_ARG;
  return launch_lrdmc(sys, w, K, d_draw, alat, 0.0, d_w, nullptr, nullptr, stream, TauArgs{d_tau_left, d_nsteps, d_eL});
}

int jqmc_branch_comb(int32_t nwalk, const double* d_w, double zeta, int32_t* d_chosen, double* d_cum, void* stream) {
  if (nwalk <= 0 || !d_w || !d_chosen || !d_cum || !(zeta >= 0.0 && zeta < 1.0)) return JQMC_E_ARG;
  k_branch_comb<<<1, 1, 0, S(stream)>>>(nwalk, d_w, d_cum);
  k_branch_search<<<(nwalk + 127) / 128, 128, 0, S(stream)>>>(nwalk, d_cum, zeta, d_chosen);
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

int jqmc_walker_gather(const jqmc_system* sys, const jqmc_walkers* src, const jqmc_walkers* dst, const int32_t* d_chosen,
                       void* stream) {
  if (!walkers_ok(sys, src) || !walkers_ok(sys, dst) || !d_chosen || src->nwalk != dst->nwalk) return JQMC_E_ARG;
  if (src->precision != dst->precision) return JQMC_E_ARG;
  const Sys& s = sys->s;
  const int W = src->nwalk;
  const long long n = s.n_up, N = s.N, A = s.det.nao, A3 = s.has_j3 ? s.j3.nao : 0;
  const int grid = 4 * 152, bs = 256;
  k_gather<double><<<grid, bs, 0, S(stream)>>>(src->r, dst->r, N * 3, d_chosen, W);
  auto tab = [&](const void* a, void* b, long long per) {
    if (is_mixed(src->precision))
      k_gather<float><<<grid, bs, 0, S(stream)>>>(static_cast<const float*>(a), static_cast<float*>(b), per, d_chosen, W);
    else
      k_gather<double><<<grid, bs, 0, S(stream)>>>(static_cast<const double*>(a), static_cast<double*>(b), per, d_chosen, W);
  };
  tab(src->G, dst->G, n * n);
  tab(src->Ginv, dst->Ginv, n * n);
  tab(src->Tup, dst->Tup, n * A);
  tab(src->Tdn, dst->Tdn, n * A);
  if (A3) tab(src->h3, dst->h3, N * A3);
  tab(src->dphi, dst->dphi, N * 4 * A);
  k_gather<double><<<grid, bs, 0, S(stream)>>>(src->ecache, dst->ecache, (N + 1) * kEC, d_chosen, W);
  if (A3) tab(src->dphi3, dst->dphi3, N * 5 * A3);
  k_gather<int><<<(W + 255) / 256, 256, 0, S(stream)>>>(src->status, dst->status, 1, d_chosen, W);
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

int jqmc_probe_fp64(int64_t iters, int32_t blocks, double* d_sink, double* flops, void* stream) {
  if (iters <= 0 || blocks <= 0 || !d_sink || !flops) return JQMC_E_ARG;
  const int bs = 256;
  k_probe_fp64<<<blocks, bs, 0, S(stream)>>>(iters, d_sink);
  *flops = 2.0 * 8.0 * (double)iters * (double)blocks * bs;
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

int jqmc_probe_fp32(int64_t iters, int32_t blocks, float* d_sink, double* flops, void* stream) {
  if (iters <= 0 || blocks <= 0 || !d_sink || !flops) return JQMC_E_ARG;
  const int bs = 256;
  k_probe_fp32<<<blocks, bs, 0, S(stream)>>>(iters, d_sink);
  *flops = 2.0 * 8.0 * (double)iters * (double)blocks * bs;
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

// ---------------------------------------------------------------------------
// Allocation-free branching.  Some callers cannot allocate device memory: a host
// code whose memory pool reserved the whole GPU at start-up (cudaMalloc would
// fail or break its accounting), or a driver loop that must not stall on the
// device synchronisation cudaMalloc may imply.  For them the comb's
// cumulative-weight scratch lives in this fixed device array instead of a
// caller buffer.  Every GPU that loads the library holds the array until the
// process exits.
static __device__ __align__(256) double g_branch_scratch[JQMC_NOALLOC_MAX_WALKERS];

static std::mutex g_noalloc_mu;
// Set-up done per device: the device address of g_branch_scratch and the unique
// ID of the CUDA context it belongs to.  cudaDeviceReset (or any other end of the
// primary context) reloads the module, possibly elsewhere; a new context has a
// new ID, so the next call repeats the set-up instead of using a stale address.
struct NoallocSetup {
  unsigned long long ctx_id = 0;
  double* ptr = nullptr;
};
static NoallocSetup g_noalloc[64];

// ID of the current context (driver entry points found through the runtime, so
// the library does not link libcuda); 0 when it cannot be read.
static unsigned long long current_context_id() {
  using GetCurrent = int (*)(void**);
  using GetId = int (*)(void*, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
    looked_up = true;
  }
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

int jqmc_branch_comb_noalloc(int32_t nwalk, const double* d_w, double zeta, int32_t* d_chosen, void* stream) {
  if (nwalk <= 0 || !d_w || !d_chosen || !(zeta >= 0.0 && zeta < 1.0)) return JQMC_E_ARG;
  if (nwalk > JQMC_NOALLOC_MAX_WALKERS) return JQMC_E_LIMIT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return JQMC_E_CUDA;
  double* scratch = nullptr;
  {
    // set-up once per device (and again after its context was replaced), with
    // that device current: the host-side symbol is only a stand-in, so the
    // kernels get the device address
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoallocSetup& su = g_noalloc[dev];
    const unsigned long long id = current_context_id();
    if (!su.ptr || id == 0 || id != su.ctx_id) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_branch_scratch) != cudaSuccess || !p) return JQMC_E_CUDA;
      su.ptr = static_cast<double*>(p);
      su.ctx_id = id;
    }
    scratch = su.ptr;
  }
  // every scratch entry the search reads is written by the cumsum first, so
  // nothing needs clearing between calls
  k_branch_comb<<<1, 1, 0, S(stream)>>>(nwalk, d_w, scratch);
  k_branch_search<<<(nwalk + 127) / 128, 128, 0, S(stream)>>>(nwalk, scratch, zeta, d_chosen);
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}


// ------------------------------------------------------------------ batches of systems
struct jqmc_batch {
  int nitem = 0, total = 0, precision = 0, nmax_up = 0, rows = 8;
  int smem_sweep = 0, smem_init = 0, smem_m = 0;
  BatchItem* d_items = nullptr;
  int* d_woff = nullptr;
};

int jqmc_batch_create(int32_t nitem, const jqmc_system* const* systems, const jqmc_walkers* walkers, jqmc_batch** out) {
  if (!out || nitem <= 0 || !systems || !walkers) return JQMC_E_ARG;
  *out = nullptr;
  std::vector<BatchItem> items(nitem);
  std::vector<int> woff(nitem);
  jqmc_batch* b = new jqmc_batch();
  b->precision = walkers[0].precision;
  int total = 0;
  bool small_ao = true;
  for (int i = 0; i < nitem; ++i) {
    const jqmc_system* sys = systems[i];
    const jqmc_walkers* w = &walkers[i];
    if (!walkers_ok(sys, w) || w->precision != b->precision) { delete b; return JQMC_E_ARG; }
    const Sys& s = sys->s;
    BatchItem& it = items[i];
    it.P = make_params(sys, w);
    it.woff = total;
    woff[i] = total;
    it.off_cand = it.P.wl.bytes;
    const int tb = tab_bytes(w);
    b->smem_sweep = std::max(b->smem_sweep, align16(it.off_cand + 2 * s.n_up * s.n_up * tb));
    it.init = init_layout(s, it.P);
    b->smem_init = std::max(b->smem_init, it.init.bytes);
    if (s.det.nao > 2048) small_ao = false;
    b->nmax_up = std::max(b->nmax_up, s.n_up);
    total += w->nwalk;
  }
  b->rows = small_ao ? 8 : 4;
  for (int i = 0; i < nitem; ++i) b->smem_m = std::max(b->smem_m, b->rows * systems[i]->s.det.nao * 8);
  b->nitem = nitem;
  b->total = total;
  if (cudaMalloc(&b->d_items, sizeof(BatchItem) * nitem) != cudaSuccess ||
      cudaMalloc(&b->d_woff, sizeof(int) * nitem) != cudaSuccess ||
      cudaMemcpy(b->d_items, items.data(), sizeof(BatchItem) * nitem, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_woff, woff.data(), sizeof(int) * nitem, cudaMemcpyHostToDevice) != cudaSuccess) {
    if (b->d_items) cudaFree(b->d_items);
    if (b->d_woff) cudaFree(b->d_woff);
    delete b;
    return JQMC_E_CUDA;
  }
  *out = b;
  return JQMC_OK;
}

int jqmc_batch_destroy(jqmc_batch* b) {
  if (!b) return JQMC_E_ARG;
  cudaDeviceSynchronize();
  if (b->d_items) cudaFree(b->d_items);
  if (b->d_woff) cudaFree(b->d_woff);
  delete b;
  return JQMC_OK;
}

int jqmc_batch_walkers(const jqmc_batch* b) { return b ? b->total : JQMC_E_ARG; }

int jqmc_vmc_sweep_batch(const jqmc_batch* b, int32_t K, const int32_t* d_idraw, const double* d_fdraw, double Dt,
                         double eps_AS, int32_t* d_accept, int32_t threads, int32_t caches, void* stream) {
  if (!b || K < 0 || !d_idraw || !d_fdraw || !d_accept) return JQMC_E_ARG;
  if (threads < 32 || threads > 256 || threads % 32) return JQMC_E_ARG;
  if (K == 0) return JQMC_OK;
  const bool mixed = is_mixed(b->precision);
  using KFn = void (*)(const BatchItem*, const int*, int, int, const int*, const double*, double, double, int*);
  const KFn fn = mixed ? (caches ? (KFn)k_vmc_sweep_batch<float, true> : (KFn)k_vmc_sweep_batch<float, false>)
                       : (caches ? (KFn)k_vmc_sweep_batch<double, true> : (KFn)k_vmc_sweep_batch<double, false>);
  int rc = launch_check((const void*)fn, b->smem_sweep);
  if (rc) return rc;
  fn<<<b->total, threads, b->smem_sweep, S(stream)>>>(b->d_items, b->d_woff, b->nitem, K, d_idraw, d_fdraw, Dt, eps_AS,
                                                      d_accept);
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

int jqmc_batch_rebuild(const jqmc_batch* b, int32_t full, void* stream) {
  if (!b) return JQMC_E_ARG;
  const int mode = full ? 0 : (kInitTablesOnly | kInitRefine | kInitJ3Table);
  if (is_mixed(b->precision)) {
    const void* fm = b->rows == 8 ? (const void*)k_rebuild_m_batch<8> : (const void*)k_rebuild_m_batch<4>;
    int rc = launch_check(fm, b->smem_m);
    if (rc) return rc;
    const dim3 grid_m(b->total, 2 * ((b->nmax_up + b->rows - 1) / b->rows));
    if (b->rows == 8) k_rebuild_m_batch<8><<<grid_m, 128, b->smem_m, S(stream)>>>(b->d_items, b->d_woff, b->nitem);
    else k_rebuild_m_batch<4><<<grid_m, 128, b->smem_m, S(stream)>>>(b->d_items, b->d_woff, b->nitem);
    rc = launch_check((const void*)k_walker_init_batch<float>, b->smem_init);
    if (rc) return rc;
    k_walker_init_batch<float><<<b->total, 128, b->smem_init, S(stream)>>>(b->d_items, b->d_woff, b->nitem,
                                                                           mode | kInitMReady);
  } else {
    int rc = launch_check((const void*)k_walker_init_batch<double>, b->smem_init);
    if (rc) return rc;
    k_walker_init_batch<double><<<b->total, 128, b->smem_init, S(stream)>>>(b->d_items, b->d_woff, b->nitem, mode);
  }
  return cudaGetLastError() == cudaSuccess ? JQMC_OK : JQMC_E_CUDA;
}

}  // extern "C"
