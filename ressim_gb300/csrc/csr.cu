// CompRowMatrix on the GPU: pattern upload, SELL-32 copy, SpMV variants
// with MTJ's semantics (mtj/src/no/uib/cipr/matrix/sparse/CompRowMatrix.java:300-394)
// and Matrices.zeroRows (mtj/src/no/uib/cipr/matrix/Matrices.java:631-652).
#include <algorithm>

#include "linalg.cuh"

namespace rsg {

namespace {

__global__ void k_sell_gather(int64_t size, const int* __restrict__ src, const double* __restrict__ val,
                              double* __restrict__ out) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= size) return;
  int s = src[q];
  out[q] = s >= 0 ? val[s] : 0.0;
}

__global__ void k_sell_to_f32(int64_t size, const double* __restrict__ in, float* __restrict__ out) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= size) return;
  out[q] = (float)in[q];
}

// mode 0: y = A x with rows whose product is exactly zero left at +0 (mult);
// mode 1: y += alpha A x (multAdd).  One thread per row over the SELL-32
// copy: loads of one slice column are 32 consecutive values, and each row
// sums its entries in CSR order, so results equal the sequential loop.
template <int MODE>
__global__ void k_spmv(int n, const int* __restrict__ slice_base, const int* __restrict__ row_len,
                       const int* __restrict__ col, const double* __restrict__ val, const double* __restrict__ x,
                       double* __restrict__ y, double alpha, const int* __restrict__ active) {
  if (active && *active != 0) return;
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  int base = slice_base[row >> 5] + (row & 31);
  int len = row_len[row];
  double d = 0;
  for (int k = 0; k < len; ++k) {
    int q = base + 32 * k;
    d += val[q] * __ldg(x + col[q]);
  }
  if (MODE == 0) y[row] = (d != 0) ? d : 0.0;
  else y[row] += alpha * d;
}

__global__ void k_spmv_f32(int n, const int* __restrict__ slice_base, const int* __restrict__ row_len,
                           const int* __restrict__ col, const float* __restrict__ val, const float* __restrict__ x,
                           float* __restrict__ y, const int* __restrict__ active) {
  if (active && *active != 0) return;
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  int base = slice_base[row >> 5] + (row & 31);
  int len = row_len[row];
  float d = 0;
  for (int k = 0; k < len; ++k) {
    int q = base + 32 * k;
    d = fmaf(val[q], __ldg(x + col[q]), d);
  }
  y[row] = d;
}

// y = A^T x (transMult, :355-372), row-sequential scatter kept deterministic
// by running one thread per column over a precomputed transpose.
__global__ void k_trans_mult(int n, const int* __restrict__ tptr, const int* __restrict__ trow,
                             const int* __restrict__ tsrc, const double* __restrict__ val,
                             const double* __restrict__ x, double* __restrict__ y) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  double acc = 0.0;
  for (int q = tptr[c]; q < tptr[c + 1]; ++q) acc += val[tsrc[q]] * x[trow[q]];
  y[c] = acc;
}

__global__ void k_zero_rows(int nrows, const int* __restrict__ rows, const int* __restrict__ rowptr,
                            const int* __restrict__ col, double* __restrict__ val, double diagonal) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrows) return;
  int r = rows[t];
  for (int q = rowptr[r]; q < rowptr[r + 1]; ++q) val[q] = (col[q] == r) ? diagonal : 0.0;
}

__global__ void k_gather_values(int64_t nnz, const int* __restrict__ src, const double* __restrict__ val,
                                double* __restrict__ out) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q < nnz) out[q] = val[src[q]];
}

}  // namespace

void CsrTranspose::update(Csr& A) {
  if (A.h_rowptr != for_rowptr || A.h_col != for_col) {
    std::vector<int> tptr(A.n + 1, 0), tcol(std::max(A.nnz, 1)), tsrc(std::max(A.nnz, 1));
    for (int q = 0; q < A.nnz; ++q) tptr[A.h_col[q] + 1]++;
    for (int c = 0; c < A.n; ++c) tptr[c + 1] += tptr[c];
    std::vector<int> fill(tptr.begin(), tptr.end() - 1);
    for (int r = 0; r < A.n; ++r)
      for (int q = A.h_rowptr[r]; q < A.h_rowptr[r + 1]; ++q) {
        const int c = A.h_col[q];
        tcol[fill[c]] = r;  // rows ascend, so each transposed row is sorted
        tsrc[fill[c]] = q;
        fill[c]++;
      }
    AT.build(A.ctx, A.n, A.nnz, tptr.data(), tcol.data());
    src.resize(std::max(A.nnz, 1));
    RSG_CUDA(cudaMemcpyAsync(src.get(), tsrc.data(), sizeof(int) * A.nnz, cudaMemcpyHostToDevice, A.ctx->stream));
    A.ctx->sync();
    for_rowptr = A.h_rowptr;
    for_col = A.h_col;
  }
  if (A.nnz)
    RSG_LAUNCH(*A.ctx, "gather_values", k_gather_values, blocks_for(A.nnz, 256), 256, 0, (int64_t)A.nnz, src.get(),
               A.val.get(), AT.val.get());
  AT.sell_dirty = true;
}

void Csr::build(Context* c, int n_, int nnz_, const int* rp, const int* cl) {
  ctx = c;
  n = n_;
  nnz = nnz_;
  if (n <= 0 || nnz < 0) throw Error(RSG_BAD_ARG, "matrix size must be positive");
  if (rp[0] != 0 || rp[n] != nnz) throw Error(RSG_BAD_ARG, "row pointers inconsistent with nnz");
  h_rowptr.assign(rp, rp + n + 1);
  h_col.assign(cl, cl + nnz);
  h_diag.assign(n, -1);
  for (int i = 0; i < n; ++i) {
    if (rp[i + 1] < rp[i]) throw Error(RSG_BAD_ARG, "row pointers must be non-decreasing");
    for (int q = rp[i]; q < rp[i + 1]; ++q) {
      if (cl[q] < 0 || cl[q] >= n) throw Error(RSG_BAD_ARG, "column index out of range");
      if (q > rp[i] && cl[q] <= cl[q - 1]) throw Error(RSG_BAD_ARG, "column indices must be sorted and unique");
      if (cl[q] == i) h_diag[i] = q;
    }
  }
  rowptr.resize(n + 1);
  col.resize(std::max(nnz, 1));
  val.resize(std::max(nnz, 1));
  diag.resize(n);
  RSG_CUDA(cudaMemcpyAsync(rowptr.get(), rp, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, ctx->stream));
  if (nnz) RSG_CUDA(cudaMemcpyAsync(col.get(), cl, sizeof(int) * nnz, cudaMemcpyHostToDevice, ctx->stream));
  RSG_CUDA(cudaMemsetAsync(val.get(), 0, sizeof(double) * std::max(nnz, 1), ctx->stream));
  RSG_CUDA(cudaMemcpyAsync(diag.get(), h_diag.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
  // SELL-32
  nslices = (n + SELL_C - 1) / SELL_C;
  std::vector<int> base(nslices + 1), len(n);
  int64_t pos = 0;
  for (int s = 0; s < nslices; ++s) {
    base[s] = (int)pos;
    int w = 0;
    for (int r = s * SELL_C; r < std::min(n, (s + 1) * SELL_C); ++r) {
      len[r] = rp[r + 1] - rp[r];
      w = std::max(w, len[r]);
    }
    pos += (int64_t)w * SELL_C;
  }
  base[nslices] = (int)pos;
  if (pos > INT32_MAX) throw Error(RSG_UNSUPPORTED, "matrix too large for 32-bit SELL offsets");
  sell_size = pos;
  std::vector<int> scol(std::max<int64_t>(pos, 1), 0), ssrc(std::max<int64_t>(pos, 1), -1);
  for (int r = 0; r < n; ++r) {
    int s = r / SELL_C, lane = r % SELL_C;
    for (int k = 0; k < len[r]; ++k) {
      int64_t q = base[s] + (int64_t)k * SELL_C + lane;
      scol[q] = cl[rp[r] + k];
      ssrc[q] = rp[r] + k;
    }
  }
  slice_base.resize(nslices + 1);
  row_len.resize(n);
  sell_col.resize(scol.size());
  sell_src.resize(ssrc.size());
  sell_val.resize(scol.size());
  RSG_CUDA(cudaMemcpyAsync(slice_base.get(), base.data(), sizeof(int) * (nslices + 1), cudaMemcpyHostToDevice,
                           ctx->stream));
  RSG_CUDA(cudaMemcpyAsync(row_len.get(), len.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
  RSG_CUDA(cudaMemcpyAsync(sell_col.get(), scol.data(), sizeof(int) * scol.size(), cudaMemcpyHostToDevice,
                           ctx->stream));
  RSG_CUDA(cudaMemcpyAsync(sell_src.get(), ssrc.data(), sizeof(int) * ssrc.size(), cudaMemcpyHostToDevice,
                           ctx->stream));
  ctx->sync();  // host vectors above go out of scope
  sell_dirty = true;
}

void Csr::refresh_sell() {
  if (!sell_dirty) return;
  RSG_LAUNCH(*ctx, "sell_gather", k_sell_gather, blocks_for(sell_size, 256), 256, 0, sell_size, sell_src.get(),
             val.get(), sell_val.get());
  sell_dirty = false;
}

void Csr::refresh_sell_f32() {
  refresh_sell();
  if (sell_valf.size() != (size_t)sell_val.size()) sell_valf.resize(sell_val.size());
  RSG_LAUNCH(*ctx, "sell_to_f32", k_sell_to_f32, blocks_for(sell_size, 256), 256, 0, sell_size, sell_val.get(),
             sell_valf.get());
}

void launch_spmv(Context& ctx, Csr& A, const double* x, double* y, const int* active) {
  A.refresh_sell();
  RSG_LAUNCH(ctx, "spmv", k_spmv<0>, blocks_for(A.n, 256), 256, 0, A.n, A.slice_base.get(), A.row_len.get(),
             A.sell_col.get(), A.sell_val.get(), x, y, 0.0, active);
}

void launch_spmv_add(Context& ctx, Csr& A, double alpha, const double* x, double* y, const int* active) {
  A.refresh_sell();
  RSG_LAUNCH(ctx, "spmv", k_spmv<1>, blocks_for(A.n, 256), 256, 0, A.n, A.slice_base.get(), A.row_len.get(),
             A.sell_col.get(), A.sell_val.get(), x, y, alpha, active);
}

void launch_spmv_f32(Context& ctx, Csr& A, const float* x, float* y, const int* active) {
  RSG_LAUNCH(ctx, "spmv_f32", k_spmv_f32, blocks_for(A.n, 256), 256, 0, A.n, A.slice_base.get(), A.row_len.get(),
             A.sell_col.get(), A.sell_valf.get(), x, y, active);
}

}  // namespace rsg

using rsg::guarded;

namespace {
struct HostVec {
  rsg::DeviceBuffer<double> a, b;
};
}  // namespace

extern "C" {

rsg_status rsg_csr_create(rsg_ctx* ctx, int32_t n, int32_t nnz, const int32_t* row_ptr, const int32_t* col,
                          rsg_csr** out) {
  if (!ctx || !out || !row_ptr || (!col && nnz > 0)) return RSG_BAD_ARG;
  *out = nullptr;
  rsg_csr* h = new rsg_csr();
  rsg_status st = guarded(&ctx->c, [&] { h->m.build(&ctx->c, n, nnz, row_ptr, col); });
  if (st != RSG_OK) {
    delete h;
    return st;
  }
  *out = h;
  return RSG_OK;
}

rsg_status rsg_csr_destroy(rsg_csr* A) {
  if (!A) return RSG_BAD_ARG;
  if (A->m.ctx) cudaStreamSynchronize(A->m.ctx->stream);
  delete A;
  return RSG_OK;
}

rsg_status rsg_csr_set_values(rsg_csr* A, const double* values) {
  if (!A || (!values && A->m.nnz)) return RSG_BAD_ARG;
  return guarded(A->m.ctx, [&] {
    if (A->m.nnz)
      RSG_CUDA(cudaMemcpyAsync(A->m.val.get(), values, sizeof(double) * A->m.nnz, cudaMemcpyHostToDevice,
                               A->m.ctx->stream));
    A->m.sell_dirty = true;
    A->m.ctx->sync();
  });
}

rsg_status rsg_csr_get_values(rsg_csr* A, double* values) {
  if (!A || (!values && A->m.nnz)) return RSG_BAD_ARG;
  return guarded(A->m.ctx, [&] {
    if (A->m.nnz)
      RSG_CUDA(cudaMemcpyAsync(values, A->m.val.get(), sizeof(double) * A->m.nnz, cudaMemcpyDeviceToHost,
                               A->m.ctx->stream));
    A->m.ctx->sync();
  });
}

static rsg_status csr_op(rsg_csr* A, int kind, double alpha, const double* x, double* y) {
  if (!A || !x || !y) return RSG_BAD_ARG;
  return guarded(A->m.ctx, [&] {
    rsg::Csr& M = A->m;
    rsg::Context& ctx = *M.ctx;
    rsg::DeviceBuffer<double> dx(M.n), dy(M.n);
    RSG_CUDA(cudaMemcpyAsync(dx.get(), x, sizeof(double) * M.n, cudaMemcpyHostToDevice, ctx.stream));
    if (kind == 1)
      RSG_CUDA(cudaMemcpyAsync(dy.get(), y, sizeof(double) * M.n, cudaMemcpyHostToDevice, ctx.stream));
    if (kind == 0) rsg::launch_spmv(ctx, M, dx.get(), dy.get(), nullptr);
    else if (kind == 1) rsg::launch_spmv_add(ctx, M, alpha, dx.get(), dy.get(), nullptr);
    else {
      // transpose map built on the host once per call (test/utility path)
      std::vector<int> tptr(M.n + 1, 0), trow(M.nnz), tsrc(M.nnz);
      for (int q = 0; q < M.nnz; ++q) tptr[M.h_col[q] + 1]++;
      for (int c = 0; c < M.n; ++c) tptr[c + 1] += tptr[c];
      std::vector<int> fill(tptr.begin(), tptr.end() - 1);
      for (int r = 0; r < M.n; ++r)
        for (int q = M.h_rowptr[r]; q < M.h_rowptr[r + 1]; ++q) {
          int c = M.h_col[q];
          trow[fill[c]] = r;
          tsrc[fill[c]] = q;
          fill[c]++;
        }
      rsg::DeviceBuffer<int> dtp(M.n + 1), dtr(std::max(M.nnz, 1)), dts(std::max(M.nnz, 1));
      RSG_CUDA(cudaMemcpyAsync(dtp.get(), tptr.data(), sizeof(int) * (M.n + 1), cudaMemcpyHostToDevice, ctx.stream));
      RSG_CUDA(cudaMemcpyAsync(dtr.get(), trow.data(), sizeof(int) * M.nnz, cudaMemcpyHostToDevice, ctx.stream));
      RSG_CUDA(cudaMemcpyAsync(dts.get(), tsrc.data(), sizeof(int) * M.nnz, cudaMemcpyHostToDevice, ctx.stream));
      RSG_LAUNCH(ctx, "trans_mult", rsg::k_trans_mult, rsg::blocks_for(M.n, 256), 256, 0, M.n, dtp.get(), dtr.get(),
                 dts.get(), M.val.get(), dx.get(), dy.get());
      ctx.sync();
    }
    RSG_CUDA(cudaMemcpyAsync(y, dy.get(), sizeof(double) * M.n, cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
  });
}

rsg_status rsg_csr_mult(rsg_csr* A, const double* x, double* y) { return csr_op(A, 0, 0.0, x, y); }
rsg_status rsg_csr_mult_add(rsg_csr* A, double alpha, const double* x, double* y) {
  return csr_op(A, 1, alpha, x, y);
}
rsg_status rsg_csr_trans_mult(rsg_csr* A, const double* x, double* y) { return csr_op(A, 2, 0.0, x, y); }

rsg_status rsg_csr_zero_rows(rsg_csr* A, double diagonal, int32_t nrows, const int32_t* rows) {
  if (!A || (nrows > 0 && !rows)) return RSG_BAD_ARG;
  return guarded(A->m.ctx, [&] {
    rsg::Csr& M = A->m;
    for (int t = 0; t < nrows; ++t) {
      if (rows[t] < 0 || rows[t] >= M.n) throw rsg::Error(RSG_BAD_ARG, "row out of range");
      if (diagonal != 0 && M.h_diag[rows[t]] < 0)
        throw rsg::Error(RSG_OUT_OF_PATTERN, "diagonal entry is not in the matrix structure");
    }
    if (nrows == 0) return;
    rsg::DeviceBuffer<int> d(nrows);
    RSG_CUDA(cudaMemcpyAsync(d.get(), rows, sizeof(int) * nrows, cudaMemcpyHostToDevice, M.ctx->stream));
    RSG_LAUNCH(*M.ctx, "zero_rows", rsg::k_zero_rows, rsg::blocks_for(nrows, 128), 128, 0, nrows, d.get(),
               M.rowptr.get(), M.col.get(), M.val.get(), diagonal);
    M.sell_dirty = true;
    M.ctx->sync();
  });
}

rsg_status rsg_csr_device_arrays(rsg_csr* A, const int32_t** row_ptr, const int32_t** col, double** values) {
  if (!A) return RSG_BAD_ARG;
  if (row_ptr) *row_ptr = A->m.rowptr.get();
  if (col) *col = A->m.col.get();
  if (values) *values = A->m.val.get();
  A->m.sell_dirty = true;  // the caller may write values
  return RSG_OK;
}

}  // extern "C"
