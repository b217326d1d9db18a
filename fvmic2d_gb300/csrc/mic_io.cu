// mic_io.cu -- marker checkpoints in fvmic2d's own field-major binary format:
// saveMarkersBinary (io.c:299-402) and restartFromMarkers (restart.c:8-125), one rank.
//
// File: int32 number of in-domain markers, float64 elapsed time, then 21 fields, each over the
// in-domain markers (cellX != -1) in the caller's array order: cpu, cellX, cellY (int32), X, Y,
// VX, VY (float64), Mat (int32), T, Tdot, eta, mu, e11, e12, Eii, s11, s22, s12, p, rho, rhodot
// (float64).  The columns are already one array per field on the device: saving is a gather
// into caller order with a compaction of the in-domain markers, one copy down and the writes.
#include <cstdio>
#include <cstring>
#include <vector>

#include "mic_internal.cuh"

using namespace mic;

namespace {

struct IoField {
  int f64, i32;  // one of them is a column index, the other -1
};
const IoField kFields[] = {{-1, C_CPU},  {-1, C_CELLX}, {-1, C_CELLY}, {C_X, -1},   {C_Y, -1},   {C_VX, -1},
                           {C_VY, -1},   {-1, C_MAT},   {C_T, -1},     {C_TDOT, -1}, {C_ETA, -1}, {C_MU, -1},
                           {C_EXX, -1},  {C_EXY, -1},   {C_EII, -1},   {C_SXX, -1}, {C_SYY, -1}, {C_SXY, -1},
                           {C_P, -1},    {C_RHO, -1},   {C_RHODOT, -1}};
constexpr int kNFields = sizeof(kFields) / sizeof(kFields[0]);

struct PackPtrs {
  const void *src[kNFields];
  void *dst[kNFields];
  int is_int[kNFields];
};

__global__ void k_io_ids(const int *__restrict__ ID, const int *__restrict__ cellX, int64_t n, int *slot_of_id,
                         int *flag) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s > n) return;
  if (s == n) {
    flag[n] = 0;
    return;
  }
  const int id = ID[s];
  slot_of_id[id] = (int)s;
  flag[id] = cellX[s] != -1;
}

// caller index k -> position pos[k] among the in-domain markers, every field
__global__ void k_io_pack(const int *__restrict__ slot_of_id, const int *__restrict__ pos, int64_t n, PackPtrs p) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n || pos[k + 1] == pos[k]) return;
  const int s = slot_of_id[k];
  const int q = pos[k];
#pragma unroll
  for (int f = 0; f < kNFields; ++f) {
    if (p.is_int[f])
      static_cast<int *>(p.dst[f])[q] = static_cast<const int *>(p.src[f])[s];
    else
      static_cast<double *>(p.dst[f])[q] = static_cast<const double *>(p.src[f])[s];
  }
}

__global__ void k_io_iota(int *ID, int64_t n) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s < n) ID[s] = (int)s;
}

int ensure_io(mic_ctx *ctx, size_t bytes) {
  if (ctx->io_bytes >= bytes) return MIC_OK;
  cudaFree(ctx->io_buf);
  ctx->io_buf = nullptr;
  ctx->io_bytes = 0;
  if (cudaMalloc(&ctx->io_buf, bytes) != cudaSuccess) return MIC_ERR_NOMEM;
  ctx->io_bytes = bytes;
  return MIC_OK;
}

size_t align8(size_t b) { return (b + 7) & ~(size_t)7; }

}  // namespace

extern "C" int mic_save_markers_binary(mic_ctx *ctx, const char *path, double elapsed_time) {
  if (!ctx || !path) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  const int64_t n = ctx->n;
  const int64_t aux_n = mic_scan_aux_ints(n + 1);
  // scratch: slot_of_id, flags/positions, scan aux, then the packed fields (n each at most)
  const size_t head = align8(sizeof(int) * (n + 1)) * 2 + align8(sizeof(int) * aux_n);
  size_t body = 0;
  for (int f = 0; f < kNFields; ++f) body += align8((kFields[f].i32 >= 0 ? 4 : 8) * (size_t)(n > 0 ? n : 1));
  int e = ensure_io(ctx, head + body);
  if (e) return e;
  unsigned char *b = static_cast<unsigned char *>(ctx->io_buf);
  int *slot_of_id = reinterpret_cast<int *>(b);
  int *pos = reinterpret_cast<int *>(b + align8(sizeof(int) * (n + 1)));
  int *aux = reinterpret_cast<int *>(b + 2 * align8(sizeof(int) * (n + 1)));
  unsigned char *packed = b + head;
  int32_t count = 0;
  if (n > 0) {
    {
      MIC_KERNEL(ctx, "k_io_ids");
      k_io_ids<<<grid_for(n + 1), kBlock, 0, ctx->stream>>>(ctx->i32[C_ID], ctx->i32[C_CELLX], n, slot_of_id, pos);
    }
    if ((e = mic_scan_exclusive(ctx, pos, n + 1, aux))) return e;
    MIC_CUDA_TRY(cudaMemcpyAsync(&count, pos + n, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  }
  PackPtrs pp;
  size_t off[kNFields], bytes[kNFields], at = 0;
  for (int f = 0; f < kNFields; ++f) {
    const bool isi = kFields[f].i32 >= 0;
    pp.is_int[f] = isi;
    pp.src[f] = isi ? (const void *)ctx->i32[kFields[f].i32] : (const void *)ctx->f64[kFields[f].f64];
    pp.dst[f] = packed + at;
    off[f] = at;
    bytes[f] = (isi ? 4 : 8) * (size_t)count;
    at += align8(bytes[f] > 0 ? bytes[f] : 1);
  }
  std::vector<unsigned char> host(at);
  if (count > 0) {
    {
      MIC_KERNEL(ctx, "k_io_pack");
      k_io_pack<<<grid_for(n), kBlock, 0, ctx->stream>>>(slot_of_id, pos, n, pp);
    }
    MIC_CUDA_TRY(cudaGetLastError());
    MIC_CUDA_TRY(cudaMemcpyAsync(host.data(), packed, at, cudaMemcpyDeviceToHost, ctx->stream));
    MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  }
  FILE *fp = fopen(path, "wb");
  if (!fp) return MIC_ERR_IO;
  bool ok = fwrite(&count, sizeof(int32_t), 1, fp) == 1 && fwrite(&elapsed_time, sizeof(double), 1, fp) == 1;
  for (int f = 0; ok && f < kNFields; ++f)
    ok = bytes[f] == 0 || fwrite(host.data() + off[f], 1, bytes[f], fp) == bytes[f];
  ok = (fclose(fp) == 0) && ok;
  return ok ? MIC_OK : MIC_ERR_IO;
}

extern "C" int mic_restart_from_markers(mic_ctx *ctx, const char *path, double *elapsed_time) {
  if (!ctx || !path) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  FILE *fp = fopen(path, "rb");
  if (!fp) return MIC_ERR_IO;
  int32_t count = 0;
  double t = 0.0;
  if (fread(&count, sizeof(int32_t), 1, fp) != 1 || fread(&t, sizeof(double), 1, fp) != 1 || count < 0) {
    fclose(fp);
    return MIC_ERR_IO;
  }
  if (count > ctx->cap) {
    fclose(fp);
    return MIC_ERR_CAPACITY;
  }
  std::vector<unsigned char> host;
  size_t off[kNFields], at = 0;
  for (int f = 0; f < kNFields; ++f) {
    off[f] = at;
    at += (kFields[f].i32 >= 0 ? 4 : 8) * (size_t)count;
  }
  host.resize(at > 0 ? at : 1);
  const bool ok = at == 0 || fread(host.data(), 1, at, fp) == at;
  fclose(fp);
  if (!ok) return MIC_ERR_IO;
  // allocateMarkers resets the new array (markers.c:15-27); the file's fields go to slots 0..count-1,
  // which is then the caller's order
  int e = mic_reset_markers(ctx);
  if (e) return e;
  for (int f = 0; f < kNFields && count > 0; ++f) {
    void *dst = kFields[f].i32 >= 0 ? (void *)ctx->i32[kFields[f].i32] : (void *)ctx->f64[kFields[f].f64];
    const size_t bytes = (kFields[f].i32 >= 0 ? 4 : 8) * (size_t)count;
    MIC_CUDA_TRY(cudaMemcpyAsync(dst, host.data() + off[f], bytes, cudaMemcpyHostToDevice, ctx->stream));
  }
  if (count > 0) {
    MIC_CUDA_TRY(cudaMemsetAsync(ctx->f64[C_SRR], 0, sizeof(double) * count, ctx->stream));
    MIC_KERNEL(ctx, "k_io_iota");
    k_io_iota<<<grid_for(count), kBlock, 0, ctx->stream>>>(ctx->i32[C_ID], count);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  ctx->n = count;
  ctx->has_grain = 0;
  ctx->gen++;
  mic_invalidate_sort(ctx);
  if ((e = mic_bin_and_sort(ctx, nullptr))) return e;  // findMarkerCells (restart.c:114)
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (elapsed_time) *elapsed_time = t;
  return MIC_OK;
}
