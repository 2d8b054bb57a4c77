// Ground-state observables of the spinless bilayer on the device, as the
// reference evaluates them from its reconstructed state psir_0
// (BLQH_without_spin/lanczos_hamiltonian.cpp:658-736):
//
//   occupation n_{alpha, j} = sum_i |psir_i|^2 (1/D_i) sum_{q < D_i} [orbital j of
//       layer alpha occupied in translate(id_i, q)]                     (:658-678)
//   pseudospin Sz = (2 <N_upper> - Ne) / (2 Ne)                         (:680-689)
//   pseudospin Sx = |sum_i sum_ql sum_n conj(psir_i) psir_j FT[ql][qr] 0.5 sign
//       / sqrt(Dl Dr)| / Ne over the single-electron interlayer moves   (:691-736)
//
// psir_0 is the reference's conjugated reconstruction (the complex conjugate
// of the ground state, see eigenstates_reconstruction :625, :632); the library
// keeps the ground state itself, so the kernel uses its conjugate to give the
// reference's numbers. Sz and the occupations only need |psi|^2.
#include <cmath>
#include <vector>

#include "sector.cuh"

namespace {

constexpr int OB_THREADS = 256;

struct ObsArgs {
  SectorIdx S;
  const uint64_t* id;
  const uint8_t* period;
  const uint32_t* map;
  const double* psi;  // ground state (dim doubles, or 2 dim interleaved)
  int64_t dim;
  int cplx, K;
};

// Per block partials: [0] <N_upper>, [1] Re Sx, [2] Im Sx, [3 .. 3 + 2 nphi) occupations.
__global__ void __launch_bounds__(OB_THREADS) k_observables(ObsArgs A, double* __restrict__ part) {
  const int nphi = A.S.nphi, nv = 3 + 2 * nphi;
  __shared__ double red[OB_THREADS / 32][3 + 2 * BLQH_MAX_NPHI];
  double acc[3 + 2 * BLQH_MAX_NPHI];
  for (int k = 0; k < nv; k++) acc[k] = 0.0;
  const uint64_t lm = (1ULL << nphi) - 1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.dim; i += (int64_t)gridDim.x * blockDim.x) {
    // psir = conj(psi)
    const double pr = A.cplx ? A.psi[2 * i] : A.psi[i];
    const double pim = A.cplx ? -A.psi[2 * i + 1] : 0.0;
    const double w = pr * pr + pim * pim;
    const uint64_t idi = A.id[i];
    acc[0] += __popcll(idi & lm) * w;
    const int Dl = A.K < 0 ? 1 : A.period[i];
    for (int ql = 0; ql < Dl; ql++) {
      int parl = 0;
      const uint64_t lb = ql == 0 ? idi : translate_bits(idi, ql, nphi, &parl);
      for (int b = 0; b < 2 * nphi; b++)
        if ((lb >> b) & 1) acc[3 + b] += w / Dl;
      // single-electron moves between the layers at orbital n
      for (int n = 0; n < nphi; n++) {
        const int nt = n + nphi;
        const uint64_t mask = (1ULL << n) | (1ULL << nt);
        const uint64_t kn = mask & lb;
        if (kn == mask || kn == 0) continue;
        const uint64_t rb0 = lb - kn + (kn ^ mask);
        const int Dr = A.K < 0 ? 1 : orbit_period(rb0, nphi);
        const int hpar = hop1_parity(lb, n, nt);
        for (int qr = 0; qr < Dr; qr++) {
          int parr = 0;
          const uint64_t rb = qr == 0 ? rb0 : inv_translate_bits(rb0, qr, nphi, &parr);
          const int64_t e = sector_index(A.S, rb);
          if (e < 0) continue;
          const uint32_t mp = A.map[e];
          if (mp == 0xFFFFFFFFu || (mp & 31u) != 0) continue;  // not itself a representative
          const int64_t j = mp >> 5;
          const double qjr = A.cplx ? A.psi[2 * j] : A.psi[j];
          const double qji = A.cplx ? -A.psi[2 * j + 1] : 0.0;
          // conj(psir_i) psir_j
          const double cr = pr * qjr + pim * qji, ci = pr * qji - pim * qjr;
          double fr = 1.0, fi = 0.0;
          if (A.K > 0) {
            const double ang = 2.0 * M_PI * (ql - qr) * A.K / nphi;
            fr = cos(ang);
            fi = sin(ang);
          }
          const double f = (((hpar + parl + parr) & 1) ? -0.5 : 0.5) / sqrt((double)(Dl * Dr));
          acc[1] += (cr * fr - ci * fi) * f;
          acc[2] += (cr * fi + ci * fr) * f;
        }
      }
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = 0; k < nv; k++) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    double s = 0;
    for (int w = 0; w < OB_THREADS / 32; w++) s += red[w][threadIdx.x];
    part[(int64_t)blockIdx.x * nv + threadIdx.x] = s;
  }
}

}  // namespace

// Sz, Sx and the 2 nphi occupations (upper layer first) of the device state psi.
void observables_impl(blqh_ctx* ctx, const blqh_basis* B, const double* psi, int cplx, double* sz, double* sx,
                      double* occ) {
  if (B->model != BLQH_MODEL_SPINLESS || !B->d_map) {
    set_error(ctx, BLQH_ERR_UNSUPPORTED, "observables: spinless bases only");
    throw BlqhError{BLQH_ERR_UNSUPPORTED, "model"};
  }
  ObsArgs A{};
  A.S = B->sx;
  A.id = B->d_id;
  A.period = B->d_period;
  A.map = B->d_map;
  A.psi = psi;
  A.dim = B->dim;
  A.cplx = cplx;
  A.K = B->sector.K;
  const int nphi = B->sector.nphi, nv = 3 + 2 * nphi;
  const int grid = grid_for(ctx, B->dim, OB_THREADS, 4);
  double* part = dalloc<double>(ctx, (size_t)grid * nv);
  std::vector<double> h((size_t)grid * nv);
  try {
    k_observables<<<grid, OB_THREADS, 0, ctx->stream>>>(A, part);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, TM_MISC);
    BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(h.data(), part, h.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  } catch (...) {
    dev_free(part);
    throw;
  }
  dev_free(part);
  std::vector<double> t(nv, 0.0);
  for (int g = 0; g < grid; g++)
    for (int k = 0; k < nv; k++) t[k] += h[(size_t)g * nv + k];
  const int nel = B->sector.nel;
  if (sz) *sz = (2.0 * t[0] - nel) / (2.0 * nel);
  if (sx) *sx = std::sqrt(t[1] * t[1] + t[2] * t[2]) / nel;
  if (occ)
    for (int k = 0; k < 2 * nphi; k++) occ[k] = t[3 + k];
}
