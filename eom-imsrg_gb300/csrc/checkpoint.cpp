// Flat operator vectors and Omega checkpoint files.
//
// vectorize / repackage (src/basic_IMSRG.f90:3929-4053) flatten an sq_op into the vector the
// reference writes to its Omega checkpoints and hands to its ODE solvers:
//   E0, fhh (A x A), fpp (P x P), fph (P x A), all column-major in full, then for every block
//   and array gam(1..6): column by column, the rows on and below the diagonal of the square
//   arrays (pppp, phph, hhhh) and every row of the rectangular ones.
// repackage fills the upper triangle of a square array from the lower one times herm.
// write_omega_checkpoint / read_omega_checkpoint (src/basic_IMSRG.f90:3215-3407) store that
// vector as a raw stream of native-endian FP64 values (Fortran access='stream', no record
// markers); the file name is the caller's (the reference derives it from its prefix and s).
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/imsrg_gb300.h"
#include "engine.h"

namespace {

int64_t neq_of(const imsrg::Layout& L) {
  int64_t n = 1 + (int64_t)L.A * L.A + (int64_t)L.P * L.P + (int64_t)L.P * L.A;
  for (int q = 0; q < L.nblocks; ++q) {
    const int64_t np = L.ncls[q][0], nb = L.ncls[q][1], nh = L.ncls[q][2];
    n += (nh * nh + nh + nb * nb + nb + np * np + np) / 2 + nb * np + nh * np + nh * nb;
  }
  return n;
}

bool square(int g) { return g == 0 || g == 3 || g == 4; }

void vectorize(const imsrg::Layout& L, const double* slab, double* v) {
  // the one-body part is the slab's own prefix
  const int64_t pre = 1 + (int64_t)L.A * L.A + (int64_t)L.P * L.P + (int64_t)L.P * L.A;
  int64_t k = 0;
  for (; k < pre; ++k) v[k] = slab[k];
  for (int q = 0; q < L.nblocks; ++q)
    for (int g = 0; g < 6; ++g) {
      const double* X = slab + L.goff[q * 6 + g];
      const int n1 = L.gn1[q * 6 + g], n2 = L.gn2[q * 6 + g];
      for (int i = 0; i < n2; ++i)
        for (int j = square(g) ? i : 0; j < n1; ++j) v[k++] = X[j + (int64_t)i * n1];
    }
}

void repackage(const imsrg::Layout& L, const double* v, int herm, double* slab) {
  const int64_t pre = 1 + (int64_t)L.A * L.A + (int64_t)L.P * L.P + (int64_t)L.P * L.A;
  int64_t k = 0;
  for (; k < pre; ++k) slab[k] = v[k];
  for (int q = 0; q < L.nblocks; ++q)
    for (int g = 0; g < 6; ++g) {
      double* X = slab + L.goff[q * 6 + g];
      const int n1 = L.gn1[q * 6 + g], n2 = L.gn2[q * 6 + g];
      for (int i = 0; i < n2; ++i)
        for (int j = square(g) ? i : 0; j < n1; ++j) {
          X[j + (int64_t)i * n1] = v[k];
          if (square(g)) X[i + (int64_t)j * n1] = v[k] * herm;
          ++k;
        }
    }
}

}  // namespace

extern "C" {

imsrg_status imsrg_neq(const imsrg_ctx* ctx, int64_t* neq) {
  if (!ctx || !neq) return IMSRG_ERR_INVALID_ARGUMENT;
  *neq = neq_of(reinterpret_cast<const Ctx*>(ctx)->L);
  return IMSRG_OK;
}

imsrg_status imsrg_vectorize_slab(const imsrg_ctx* ctx, const double* slab, double* vec) {
  if (!ctx || !slab || !vec) return IMSRG_ERR_INVALID_ARGUMENT;
  vectorize(reinterpret_cast<const Ctx*>(ctx)->L, slab, vec);
  return IMSRG_OK;
}

imsrg_status imsrg_repackage_slab(const imsrg_ctx* ctx, const double* vec, int32_t herm, double* slab) {
  if (!ctx || !vec || !slab || (herm != 1 && herm != -1)) return IMSRG_ERR_INVALID_ARGUMENT;
  repackage(reinterpret_cast<const Ctx*>(ctx)->L, vec, herm, slab);
  return IMSRG_OK;
}

imsrg_status imsrg_write_omega_checkpoint(imsrg_ctx* ctx, const imsrg_op* G, const char* path) {
  if (!ctx) return IMSRG_ERR_INVALID_ARGUMENT;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  if (!G || G->owner != c || !path) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_write_omega_checkpoint");
  const imsrg::Layout& L = c->L;
  std::vector<double> slab((size_t)L.slab), v((size_t)neq_of(L));
  imsrg_status st = imsrg_op_download_slab(ctx, G, slab.data());
  if (st != IMSRG_OK) return st;
  vectorize(L, slab.data(), v.data());
  FILE* f = std::fopen(path, "wb");
  if (!f) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, std::string("cannot open for writing: ") + path);
  const size_t w = std::fwrite(v.data(), sizeof(double), v.size(), f);
  const int cl = std::fclose(f);
  if (w != v.size() || cl != 0) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, std::string("short write: ") + path);
  return IMSRG_OK;
}

imsrg_status imsrg_read_omega_checkpoint(imsrg_ctx* ctx, imsrg_op* G, const char* path) {
  if (!ctx) return IMSRG_ERR_INVALID_ARGUMENT;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  if (!G || G->owner != c || !path) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_read_omega_checkpoint");
  const imsrg::Layout& L = c->L;
  std::vector<double> v((size_t)neq_of(L)), slab((size_t)L.slab, 0.0);
  FILE* f = std::fopen(path, "rb");
  if (!f) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, std::string("cannot open: ") + path);
  const size_t r = std::fread(v.data(), sizeof(double), v.size(), f);
  const bool extra = std::fgetc(f) != EOF;
  std::fclose(f);
  if (r != v.size() || extra)
    return c->fail(IMSRG_ERR_MISMATCH, std::string("checkpoint size does not match this basis: ") + path);
  repackage(L, v.data(), G->herm, slab.data());
  return imsrg_op_upload_slab(ctx, G, slab.data());
}

}  // extern "C"
