// C ABI: metadata (A, I, Ad, A1, I1, Ad1) installed from the host or built on the device
// (include/leap_gb300.h: leap_set_metadata, leap_build_metadata, leap_get_metadata_matrix).
#include "leap_internal.h"
#include "kernels_metadata.cuh"

namespace leapabi {

// Install a metadata set: constants, sparse rows of A, I1, and Ad / Ad1 from host
// memory (kind HostToDevice) or device memory (DeviceToDevice).
int install_metadata(leap_ctx* ctx, const leap_constants* k, const std::vector<int4>& arow,
                     const std::vector<double2>& aval, int32_t A_cols, const int32_t* I1, int32_t A1_rows,
                     const double* Ad, const double* Ad1, cudaMemcpyKind kind) {
  const int32_t A_rows = static_cast<int32_t>(arow.size());
  for (int32_t i = 0; i + 1 < A1_rows; ++i) {
    const int64_t idx = I1[i] < 0 ? static_cast<int64_t>(I1[i]) + k->nbaselines : I1[i];
    if (idx < 0 || idx >= static_cast<int64_t>(k->nbaselines))
      return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "I1 index out of range");
  }
  Metadata& md = ctx->md;
  md.set = false;
  md.k = *k;
  md.S = A_cols;
  md.Arows = A_rows;
  md.A1rows = A1_rows;
  md.Kpad = ((A_rows + 127) / 128) * 128;
  const size_t nI1 = static_cast<size_t>(std::max(A1_rows - 1, 0));
  const size_t nad = static_cast<size_t>(A_cols) * A_rows;
  LEAP_CUDA(md.I1.ensure(sizeof(int32_t) * std::max<size_t>(nI1, 1)), "alloc I1");
  LEAP_CUDA(md.Ad1.ensure(sizeof(double) * A_cols * A1_rows), "alloc Ad1");
  LEAP_CUDA(md.Ad.ensure(sizeof(double) * nad), "alloc Ad");
  LEAP_CUDA(md.Ad_f32.ensure(sizeof(float) * nad), "alloc Ad f32");
  LEAP_CUDA(md.arow.ensure(sizeof(int4) * A_rows), "alloc A rows");
  LEAP_CUDA(md.arow_val.ensure(sizeof(double2) * A_rows), "alloc A values");
  if (nI1) LEAP_CUDA(cudaMemcpy(md.I1.ptr, I1, sizeof(int32_t) * nI1, cudaMemcpyHostToDevice), "upload I1");
  if (Ad1 != md.Ad1.as<double>())
    LEAP_CUDA(cudaMemcpy(md.Ad1.ptr, Ad1, sizeof(double) * A_cols * A1_rows, kind), "upload Ad1");
  if (Ad != md.Ad.as<double>()) LEAP_CUDA(cudaMemcpy(md.Ad.ptr, Ad, sizeof(double) * nad, kind), "upload Ad");
  to_float<<<grid_1d(static_cast<int64_t>(nad), 256), 256, 0, ctx->stream>>>(md.Ad.as<double>(), nad, md.Ad_f32.as<float>());
  LEAP_CUDA(cudaMemcpy(md.arow.ptr, arow.data(), sizeof(int4) * A_rows, cudaMemcpyHostToDevice), "upload A rows");
  LEAP_CUDA(cudaMemcpy(md.arow_val.ptr, aval.data(), sizeof(double2) * A_rows, cudaMemcpyHostToDevice), "upload A vals");
  // A^T over the rows n < |I| (the rows dInt reads), compressed by column, for the adjoint.
  {
    const int32_t nI = A_rows - 1;
    std::vector<int32_t> ptr(A_cols + 1, 0);
    for (int32_t n = 0; n < nI; ++n) {
      ++ptr[arow[n].x + 1];
      if (arow[n].y != arow[n].x) ++ptr[arow[n].y + 1];
    }
    for (int32_t c = 0; c < A_cols; ++c) ptr[c + 1] += ptr[c];
    std::vector<int32_t> idx(std::max(ptr[A_cols], 1));
    std::vector<double> val(std::max(ptr[A_cols], 1));
    std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
    for (int32_t n = 0; n < nI; ++n) {
      idx[fill[arow[n].x]] = n;
      val[fill[arow[n].x]++] = aval[n].x;
      if (arow[n].y != arow[n].x) {
        idx[fill[arow[n].y]] = n;
        val[fill[arow[n].y]++] = aval[n].y;
      }
    }
    LEAP_CUDA(md.at_ptr.ensure(sizeof(int32_t) * ptr.size()), "alloc A^T");
    LEAP_CUDA(md.at_idx.ensure(sizeof(int32_t) * idx.size()), "alloc A^T");
    LEAP_CUDA(md.at_val.ensure(sizeof(double) * val.size()), "alloc A^T");
    LEAP_CUDA(cudaMemcpy(md.at_ptr.ptr, ptr.data(), sizeof(int32_t) * ptr.size(), cudaMemcpyHostToDevice), "upload A^T");
    LEAP_CUDA(cudaMemcpy(md.at_idx.ptr, idx.data(), sizeof(int32_t) * idx.size(), cudaMemcpyHostToDevice), "upload A^T");
    LEAP_CUDA(cudaMemcpy(md.at_val.ptr, val.data(), sizeof(double) * val.size(), cudaMemcpyHostToDevice), "upload A^T");
  }
  // Ad split into TF32 hi/lo and packed once for the tensor-core contraction.
  md.tc_mtiles = (A_cols + kTcM - 1) / kTcM;
  md.tc_kblocks = md.Kpad / kTcKB;
  LEAP_CUDA(md.Ad_tc.ensure(static_cast<size_t>(md.tc_mtiles) * md.tc_kblocks * 2 * kTcBlockBytesA), "alloc packed Ad");
  tc_pack_ad<<<grid_1d(static_cast<int64_t>(md.tc_mtiles) * kTcM * md.tc_kblocks * kTcKB, 256), 256, 0, ctx->stream>>>(
      md.Ad.as<double>(), A_cols, A_rows, md.tc_mtiles, md.tc_kblocks, md.Ad_tc.as<float>());
  LEAP_CUDA(cudaGetLastError(), "pack Ad");
  LEAP_CUDA(cudaStreamSynchronize(ctx->stream), "pack Ad");
  md.set = true;
  return LEAP_OK;
}

// Sparse rows (column order) of a column-major dense phase matrix.
int sparse_rows(leap_ctx* ctx, const double* A, int32_t A_rows, int32_t A_cols, std::vector<int4>& arow,
                std::vector<double2>& aval) {
  arow.resize(A_rows);
  aval.resize(A_rows);
  for (int32_t r = 0; r < A_rows; ++r) {
    int nz = 0;
    int cidx[2] = {0, 0};
    double v[2] = {0.0, 0.0};
    for (int32_t c = 0; c < A_cols; ++c) {
      const double x = A[r + static_cast<size_t>(A_rows) * c];
      if (x != 0.0) {
        if (nz == 2) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "A row has more than two non-zeros");
        cidx[nz] = c;
        v[nz] = x;
        ++nz;
      }
    }
    arow[r] = make_int4(cidx[0], nz > 1 ? cidx[1] : cidx[0], 0, 0);
    aval[r] = make_double2(v[0], v[1]);
  }
  return LEAP_OK;
}

// Pseudo-inverse of a phase matrix on the device (see kernels_metadata.cuh) into
// Ad_out (device, S x Arows column-major).  Returns LEAP_OK, or LEAP_ERR_NOT_READY
// when the Gram matrix is not safely invertible (the caller then uses the host path).
int device_pinv(leap_ctx* ctx, const std::vector<int4>& arow, const std::vector<double2>& aval, int32_t S,
                double* Ad_out) {
  const int32_t m = static_cast<int32_t>(arow.size());
  // Exact integer Gram matrix and the columns A uses.
  std::vector<double> G(static_cast<size_t>(S) * S, 0.0);
  for (int32_t r = 0; r < m; ++r) {
    const int c[2] = {arow[r].x, arow[r].y};
    const double v[2] = {aval[r].x, aval[r].y};
    const int nz = c[1] != c[0] ? 2 : 1;
    for (int a = 0; a < nz; ++a)
      for (int b = 0; b < nz; ++b) G[static_cast<size_t>(c[a]) * S + c[b]] += v[a] * v[b];
  }
  std::vector<int32_t> cmp(S, -1);
  int n = 0;
  for (int32_t c = 0; c < S; ++c)
    if (G[static_cast<size_t>(c) * S + c] != 0.0) cmp[c] = n++;
  if (n == 0) return LEAP_ERR_NOT_READY;
  std::vector<double> Gc(static_cast<size_t>(n) * n);
  double gf = 0.0;
  for (int32_t i = 0; i < S; ++i)
    for (int32_t j = 0; j < S; ++j)
      if (cmp[i] >= 0 && cmp[j] >= 0) {
        const double x = G[static_cast<size_t>(i) * S + j];
        Gc[static_cast<size_t>(cmp[i]) * n + cmp[j]] = x;
        gf += x * x;
      }
  const size_t nn = static_cast<size_t>(n) * n;
  DeviceBuffer dG, dX, dR, dY, dr, df, dbad, dnorm, dcmp, darow, daval;
  struct Release {  // scratch goes on every return path
    std::initializer_list<DeviceBuffer*> bufs;
    ~Release() {
      for (DeviceBuffer* b : bufs) b->release();
    }
  } release_all{{&dG, &dX, &dR, &dY, &dr, &df, &dbad, &dnorm, &dcmp, &darow, &daval}};
  LEAP_CUDA(dG.ensure(sizeof(double) * nn), "alloc pinv");
  LEAP_CUDA(dX.ensure(sizeof(double) * nn), "alloc pinv");
  LEAP_CUDA(dR.ensure(sizeof(double) * nn), "alloc pinv");
  LEAP_CUDA(dY.ensure(sizeof(double) * nn), "alloc pinv");
  LEAP_CUDA(dr.ensure(sizeof(double) * n), "alloc pinv");
  LEAP_CUDA(df.ensure(sizeof(double) * n), "alloc pinv");
  LEAP_CUDA(dbad.ensure(sizeof(int)), "alloc pinv");
  LEAP_CUDA(dnorm.ensure(sizeof(double)), "alloc pinv");
  LEAP_CUDA(dcmp.ensure(sizeof(int32_t) * S), "alloc pinv");
  LEAP_CUDA(darow.ensure(sizeof(int4) * m), "alloc pinv");
  LEAP_CUDA(daval.ensure(sizeof(double2) * m), "alloc pinv");
  cudaStream_t s = ctx->stream;
  LEAP_CUDA(cudaMemcpyAsync(dG.ptr, Gc.data(), sizeof(double) * nn, cudaMemcpyHostToDevice, s), "upload G");
  LEAP_CUDA(cudaMemcpyAsync(dX.ptr, dG.ptr, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s), "copy G");
  LEAP_CUDA(cudaMemcpyAsync(dcmp.ptr, cmp.data(), sizeof(int32_t) * S, cudaMemcpyHostToDevice, s), "upload columns");
  LEAP_CUDA(cudaMemcpyAsync(darow.ptr, arow.data(), sizeof(int4) * m, cudaMemcpyHostToDevice, s), "upload rows");
  LEAP_CUDA(cudaMemcpyAsync(daval.ptr, aval.data(), sizeof(double2) * m, cudaMemcpyHostToDevice, s), "upload rows");
  LEAP_CUDA(cudaMemsetAsync(dbad.ptr, 0, sizeof(int), s), "clear");
  const int ug = grid_1d(static_cast<int64_t>(nn), 256);
  for (int k = 0; k < n; ++k) {
    gj_pivot<<<1, 512, 0, s>>>(dX.as<double>(), n, k, dr.as<double>(), df.as<double>(), dbad.as<int>());
    gj_update<<<ug, 256, 0, s>>>(dX.as<double>(), n, k, dr.as<double>(), df.as<double>());
  }
  for (int step = 0; step < 2; ++step) {
    residual_dd<<<ug, 256, 0, s>>>(dX.as<double>(), dG.as<double>(), n, dR.as<double>());
    refine_apply<<<ug, 256, 0, s>>>(dX.as<double>(), dR.as<double>(), n, dY.as<double>());
    std::swap(dX.ptr, dY.ptr);
    std::swap(dX.bytes, dY.bytes);
  }
  sum_squares<<<1, 256, 0, s>>>(dX.as<double>(), static_cast<int64_t>(nn), dnorm.as<double>());
  LEAP_CUDA(cudaGetLastError(), "pinv kernels");
  int bad = 0;
  double xf2 = 0.0;
  LEAP_CUDA(cudaMemcpyAsync(&bad, dbad.ptr, sizeof(int), cudaMemcpyDeviceToHost, s), "read pivot check");
  LEAP_CUDA(cudaMemcpyAsync(&xf2, dnorm.ptr, sizeof(double), cudaMemcpyDeviceToHost, s), "read norm");
  LEAP_CUDA(cudaStreamSynchronize(s), "pinv");
  // lambda_min(G) >= 1/||X||_F; the reference truncates at max(m,n)*eps*sigma_0 on sigma,
  // i.e. at about max(m,n)*eps*lambda_0 on lambda (lambda_0 <= ||G||_F).  Keep a margin of 1e3.
  const double tol = static_cast<double>(std::max(m, S)) * std::numeric_limits<double>::epsilon() * std::sqrt(gf);
  if (bad || !(xf2 > 0.0) || !std::isfinite(xf2) || 1.0 / std::sqrt(xf2) <= 1e3 * tol) return LEAP_ERR_NOT_READY;
  assemble_pinv<<<grid_1d(static_cast<int64_t>(S) * m, 256), 256, 0, s>>>(
      dX.as<double>(), n, dcmp.as<int32_t>(), darow.as<int4>(), daval.as<double2>(), S, m, Ad_out);
  LEAP_CUDA(cudaGetLastError(), "assemble pinv");
  LEAP_CUDA(cudaStreamSynchronize(s), "assemble pinv");
  return LEAP_OK;
}

}  // namespace leapabi

extern "C" {

int32_t leap_set_metadata(leap_ctx* ctx, const leap_constants* k, const double* A, int32_t A_rows, int32_t A_cols,
                          const int32_t* I, const double* Ad, const double* A1, int32_t A1_rows, const int32_t* I1,
                          const double* Ad1) {
  if (!ctx || !k || !A || !Ad || !A1 || !I1 || !Ad1) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  (void)I;
  if (A_rows < 1 || A_cols < 1 || A1_rows < 1) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "empty phase matrix");
  if (k->nbaselines == 0) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "nbaselines must be positive");
  if (static_cast<int64_t>(A_rows) - 1 > static_cast<int64_t>(k->nbaselines))
    return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "A has more rows than baselines + 1");
  DeviceGuard g(ctx->device);
  std::vector<int4> arow;
  std::vector<double2> aval;
  int rc = sparse_rows(ctx, A, A_rows, A_cols, arow, aval);
  if (rc != LEAP_OK) return rc;
  return install_metadata(ctx, k, arow, aval, A_cols, I1, A1_rows, Ad, Ad1, cudaMemcpyHostToDevice);
}

int32_t leap_build_metadata(leap_ctx* ctx, const leap_constants* k, const int32_t* a1, const int32_t* a2,
                            const uint8_t* fg, int32_t nbl, int32_t* used_host_path) {
  if (!ctx || !k || !a1 || !a2 || !fg) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  if (nbl <= 0 || static_cast<uint32_t>(nbl) != k->nbaselines)
    return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "nbl must equal constants.nbaselines");
  DeviceGuard g(ctx->device);
  std::string err;
  std::vector<SparseRow> sA, sA1;
  std::vector<int32_t> I, I1;
  int32_t cols = 0, cols1 = 0;
  int rc = phase_matrix_sparse(a1, a2, fg, nbl, -1, sA, I, cols, err);
  if (rc != LEAP_OK) return fail(ctx, rc, err);
  rc = phase_matrix_sparse(a1, a2, fg, nbl, static_cast<int32_t>(k->referenceAntenna), sA1, I1, cols1, err);
  if (rc != LEAP_OK) return fail(ctx, rc, err);
  auto to_dev = [](const std::vector<SparseRow>& r, std::vector<int4>& ar, std::vector<double2>& av) {
    ar.resize(r.size());
    av.resize(r.size());
    for (size_t i = 0; i < r.size(); ++i) {
      ar[i] = make_int4(r[i].c0, r[i].c1, 0, 0);
      av[i] = make_double2(r[i].v0, r[i].v1);
    }
  };
  std::vector<int4> arow, arow1;
  std::vector<double2> aval, aval1;
  to_dev(sA, arow, aval);
  to_dev(sA1, arow1, aval1);
  const int32_t A_rows = static_cast<int32_t>(arow.size()), A1_rows = static_cast<int32_t>(arow1.size());
  Metadata& md = ctx->md;
  md.set = false;
  LEAP_CUDA(md.Ad.ensure(sizeof(double) * cols * A_rows), "alloc Ad");
  LEAP_CUDA(md.Ad1.ensure(sizeof(double) * cols * A1_rows), "alloc Ad1");
  int host = 0;
  for (int which = 0; which < 2; ++which) {
    const auto& ar = which == 0 ? arow : arow1;
    const auto& av = which == 0 ? aval : aval1;
    double* out = which == 0 ? md.Ad.as<double>() : md.Ad1.as<double>();
    rc = device_pinv(ctx, ar, av, cols, out);
    if (rc == LEAP_ERR_NOT_READY) {
      // Rank-deficient or ill-conditioned Gram matrix: the SVD-style host path, as the reference truncates.
      host |= 1 << which;
      const int32_t rows = static_cast<int32_t>(ar.size());
      std::vector<double> A(static_cast<size_t>(rows) * cols, 0.0), Ad(static_cast<size_t>(rows) * cols);
      for (int32_t r = 0; r < rows; ++r) {
        A[r + static_cast<size_t>(rows) * ar[r].x] = av[r].x;
        if (ar[r].y != ar[r].x) A[r + static_cast<size_t>(rows) * ar[r].y] = av[r].y;
      }
      rc = pseudo_inverse(A.data(), rows, cols, Ad.data(), err);
      if (rc != LEAP_OK) return fail(ctx, rc, err);
      LEAP_CUDA(cudaMemcpy(out, Ad.data(), sizeof(double) * Ad.size(), cudaMemcpyHostToDevice), "upload Ad");
    } else if (rc != LEAP_OK) {
      return rc;
    }
  }
  if (used_host_path) *used_host_path = host;
  return install_metadata(ctx, k, arow, aval, cols, I1.data(), A1_rows, md.Ad.as<double>(), md.Ad1.as<double>(),
                          cudaMemcpyDeviceToDevice);
}

int32_t leap_get_metadata_matrix(leap_ctx* ctx, int32_t which, double* out, int64_t capacity, int32_t* rows_out,
                                 int32_t* cols_out) {
  if (!ctx) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL context");
  if (!ctx->md.set) return fail(ctx, LEAP_ERR_NOT_READY, "metadata not set");
  const Metadata& md = ctx->md;
  if (which != 0 && which != 1) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "which must be 0 (Ad) or 1 (Ad1)");
  const int32_t cols = which == 0 ? md.Arows : md.A1rows;
  if (rows_out) *rows_out = md.S;
  if (cols_out) *cols_out = cols;
  if (!out) return LEAP_OK;
  const int64_t n = static_cast<int64_t>(md.S) * cols;
  if (capacity < n) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "output capacity too small");
  DeviceGuard g(ctx->device);
  LEAP_CUDA(cudaMemcpy(out, which == 0 ? md.Ad.ptr : md.Ad1.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost), "copy Ad");
  return LEAP_OK;
}

}  // extern "C"
