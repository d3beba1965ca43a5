// On-disk CSR matrices in the layout of CPP/io/matrix_reader.cpp:8-50:
//   <prefix>_row_ptr.bin          int32, rows + 1 entries
//   <prefix>_col_ind.bin          int32, nnz entries, 0-based
//   <prefix>_values.bin           float64, nnz entries
//   <prefix>_singular_values.bin  float64 (the matrix's known spectrum, for checking a solve)
// Element counts come from the file sizes (matrix_reader.cpp:55-66); the column count is the largest
// column index + 1 (matrix_reader.cpp:40-43).  A missing file is OFRR_ERR_FILE_NOT_FOUND; an empty
// one, a size that is not a whole number of elements, or col_ind / values of different lengths is
// OFRR_ERR_INVALID_FORMAT (the reference throws on the empty cases).  Unlike the reference, the
// structure is validated before use -- row_ptr[0] = 0, non-decreasing, row_ptr[rows] = nnz,
// col_ind >= 0 -- because the sparse kernels index memory with it: a malformed file is an error
// here, not an out-of-range access later.
// Device loads stream each file through two pinned staging buffers (one cudaMemcpyAsync per chunk on
// the context's stream, the next chunk read from disk while the previous one copies) and validate on
// the GPU in one pass over row_ptr and col_ind (grid-stride, flags and the column maximum by atomics).
#include <cstdio>
#include <string>

#include "ofrr_internal.cuh"

namespace ofrr {
namespace {

constexpr size_t kStageBytes = size_t(16) << 20;

// size in bytes of a file, -1 when it cannot be opened
long long file_bytes(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return -1;
  long long n = -1;
  if (std::fseek(f, 0, SEEK_END) == 0) n = (long long)std::ftell(f);
  std::fclose(f);
  return n;
}

// element count of a file of elements of `es` bytes (status in *st)
int64_t file_count(const std::string& path, size_t es, int* st) {
  const long long b = file_bytes(path);
  if (b < 0) {
    *st = OFRR_ERR_FILE_NOT_FOUND;
    return 0;
  }
  if (b == 0 || (size_t)b % es != 0) {
    *st = OFRR_ERR_INVALID_FORMAT;
    return 0;
  }
  *st = OFRR_SUCCESS;
  return (int64_t)((size_t)b / es);
}

int csr_sizes(const char* prefix, int64_t* nrows, int64_t* nnz) {
  const std::string p(prefix);
  int st;
  const int64_t nip = file_count(p + "_row_ptr.bin", 4, &st);
  if (st) return st;
  const int64_t nix = file_count(p + "_col_ind.bin", 4, &st);
  if (st) return st;
  const int64_t nv = file_count(p + "_values.bin", 8, &st);
  if (st) return st;
  if (nix != nv || nip - 1 > 0x7fffffffLL || nix > 0x7fffffffLL) return OFRR_ERR_INVALID_FORMAT;
  *nrows = nip - 1;
  *nnz = nix;
  return OFRR_SUCCESS;
}

// whole file into host memory
int read_host(const std::string& path, void* dst, size_t bytes) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return OFRR_ERR_FILE_NOT_FOUND;
  const size_t got = std::fread(dst, 1, bytes, f);
  std::fclose(f);
  return got == bytes ? OFRR_SUCCESS : OFRR_ERR_INVALID_FORMAT;
}

// whole file into device memory through the two pinned staging buffers
int read_device(ofrr_ctx* ctx, const std::string& path, void* dst, size_t bytes, char* stage[2], cudaEvent_t ev[2]) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return OFRR_ERR_FILE_NOT_FOUND;
  int st = OFRR_SUCCESS;
  size_t off = 0;
  for (int c = 0; off < bytes; ++c) {
    const int s = c & 1;
    if (cudaEventSynchronize(ev[s]) != cudaSuccess) {  // the previous copy out of this buffer is done
      st = OFRR_ERR_CUDA_SYNC;
      break;
    }
    const size_t n = std::min(kStageBytes, bytes - off);
    if (std::fread(stage[s], 1, n, f) != n) {
      st = OFRR_ERR_INVALID_FORMAT;
      break;
    }
    if (cudaMemcpyAsync((char*)dst + off, stage[s], n, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaEventRecord(ev[s], ctx->stream) != cudaSuccess) {
      st = OFRR_ERR_CUDA_MEMORY;
      break;
    }
    off += n;
  }
  std::fclose(f);
  return st;
}

// out[0]: structure errors (bit 0 row_ptr[0], bit 1 decreasing row_ptr, bit 2 row_ptr[rows] != nnz,
// bit 3 negative column index); out[1]: the largest column index (-1 without entries)
__global__ void k_csr_check(int64_t nrows, int64_t nnz, const int32_t* __restrict__ ip, const int32_t* __restrict__ ix,
                            int* __restrict__ out) {
  int bad = 0, mx = -1;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= nrows; i += stride) {
    const int v = ip[i];
    if (i == 0 && v != 0) bad |= 1;
    if (i > 0 && v < ip[i - 1]) bad |= 2;
    if (i == nrows && (int64_t)v != nnz) bad |= 4;
  }
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += stride) {
    const int c = ix[k];
    if (c < 0) bad |= 8;
    mx = max(mx, c);
  }
  for (int o = 16; o > 0; o >>= 1) {
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if ((threadIdx.x & 31) == 0) {
    if (bad) atomicOr(out, bad);
    atomicMax(out + 1, mx);
  }
}

int check_host(int64_t nrows, int64_t nnz, const int32_t* ip, const int32_t* ix, int64_t* ncols) {
  if (ip[0] != 0 || (int64_t)ip[nrows] != nnz) return OFRR_ERR_INVALID_FORMAT;
  for (int64_t i = 1; i <= nrows; ++i)
    if (ip[i] < ip[i - 1]) return OFRR_ERR_INVALID_FORMAT;
  int mx = -1;
  for (int64_t k = 0; k < nnz; ++k) {
    if (ix[k] < 0) return OFRR_ERR_INVALID_FORMAT;
    mx = std::max(mx, ix[k]);
  }
  *ncols = (int64_t)mx + 1;
  return OFRR_SUCCESS;
}

}  // namespace
}  // namespace ofrr

using namespace ofrr;

extern "C" int ofrr_csr_file_sizes(const char* prefix, int64_t* nrows, int64_t* nnz) {
  if (!prefix || !nrows || !nnz) return OFRR_ERR_INVALID_ARGUMENT;
  return csr_sizes(prefix, nrows, nnz);
}

extern "C" int ofrr_csr_file_read(ofrr_ctx* ctx, const char* prefix, int64_t nrows, int64_t nnz, int32_t* indptr,
                                  int32_t* indices, double* values, int64_t* ncols, int on_device) {
  if (!prefix || !indptr || !indices || !values || !ncols || (on_device && !ctx)) return OFRR_ERR_INVALID_ARGUMENT;
  int64_t fr = 0, fz = 0;
  OFRR_TRY(csr_sizes(prefix, &fr, &fz));
  if (fr != nrows || fz != nnz) return OFRR_ERR_INVALID_ARGUMENT;  // buffers sized for another matrix
  const std::string p(prefix);
  const size_t bip = sizeof(int32_t) * (size_t)(nrows + 1), bix = sizeof(int32_t) * (size_t)nnz,
               bv = sizeof(double) * (size_t)nnz;
  if (!on_device) {
    OFRR_TRY(read_host(p + "_row_ptr.bin", indptr, bip));
    OFRR_TRY(read_host(p + "_col_ind.bin", indices, bix));
    OFRR_TRY(read_host(p + "_values.bin", values, bv));
    return check_host(nrows, nnz, indptr, indices, ncols);
  }
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  int* dflags = ws_get<int>(ctx, 2, &st);
  if (!dflags) return st;
  char* stage[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  for (int s = 0; s < 2 && st == OFRR_SUCCESS; ++s) {
    if (cudaHostAlloc((void**)&stage[s], kStageBytes, cudaHostAllocDefault) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev[s], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventRecord(ev[s], ctx->stream) != cudaSuccess)
      st = OFRR_ERR_CUDA_MEMORY;
  }
  if (st == OFRR_SUCCESS) st = read_device(ctx, p + "_row_ptr.bin", indptr, bip, stage, ev);
  if (st == OFRR_SUCCESS) st = read_device(ctx, p + "_col_ind.bin", indices, bix, stage, ev);
  if (st == OFRR_SUCCESS) st = read_device(ctx, p + "_values.bin", values, bv, stage, ev);
  int hflags[2] = {0, -1};
  if (st == OFRR_SUCCESS &&
      cudaMemcpyAsync(dflags, hflags, sizeof hflags, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
    st = OFRR_ERR_CUDA_MEMORY;
  if (st == OFRR_SUCCESS) {
    const int64_t work = std::max<int64_t>(nrows + 1, nnz);
    const unsigned grid = (unsigned)std::min<int64_t>((work + 255) / 256, 152 * 8);
    k_csr_check<<<grid, 256, 0, ctx->stream>>>(nrows, nnz, indptr, indices, dflags);
    st = after_launch(ctx, "k_csr_check");
  }
  if (st == OFRR_SUCCESS &&
      cudaMemcpyAsync(hflags, dflags, sizeof hflags, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess)
    st = OFRR_ERR_CUDA_MEMORY;
  if (st == OFRR_SUCCESS) st = sync_and_check(ctx);
  if (st == OFRR_SUCCESS) {
    if (hflags[0] != 0) st = OFRR_ERR_INVALID_FORMAT;
    else *ncols = (int64_t)hflags[1] + 1;
  }
  for (int s = 0; s < 2; ++s) {  // staging buffers go once their last copy is done
    if (ev[s]) cudaEventSynchronize(ev[s]);
    if (stage[s]) cudaFreeHost(stage[s]);
    if (ev[s]) cudaEventDestroy(ev[s]);
  }
  return st;
}

extern "C" int ofrr_read_singular_values(const char* prefix, int64_t* count, double* values) {
  if (!prefix || !count) return OFRR_ERR_INVALID_ARGUMENT;
  const std::string path = std::string(prefix) + "_singular_values.bin";
  int st;
  const int64_t n = file_count(path, 8, &st);
  if (st) return st;
  if (values) {
    if (*count < n) return OFRR_ERR_INVALID_ARGUMENT;  // *count: capacity of values on entry
    OFRR_TRY(read_host(path, values, sizeof(double) * (size_t)n));
  }
  *count = n;
  return OFRR_SUCCESS;
}
