// Host-only check of the split Gram's staging layout (ozg_layout in
// blopex_gb300/csrc/oz_gram.cu): no GPU is used.  The kernel source is
// included for its host code; the library functions it calls are stubbed
// and the CUDA driver's tensor-map encoder is replaced by one that checks its
// arguments the way the driver documents them (16-byte aligned base and
// strides, box dimensions of at most 256) and succeeds, except on every fifth
// call (the fallback to per-column copies).
//
// For random L and Q blocks -- contiguous with a padded leading dimension,
// masked (columns skipped), scattered, merged from several blocks, FP32 and
// FP64, short and long -- every tile's layout must keep every column inside
// the staging buffer, no two columns overlapping, every TMA tile 128-byte
// aligned with its columns at exactly the tile's stride, every map covering
// one run of equally spaced, non-overlapping columns of one block, and map
// slots local to the tile.  Prints "ok" and exits 0, or names the failure.
#include "oz_gram.cu"

#include <stdarg.h>
#include <stdio.h>

#include <algorithm>
#include <random>
#include <utility>
#include <vector>

static long g_encoder_calls = 0;

static CUresult check_encoder(CUtensorMap* m, CUtensorMapDataType, cuuint32_t rank, void* base,
                              const cuuint64_t* dims, const cuuint64_t* strides, const cuuint32_t* box,
                              const cuuint32_t* es, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill)
{
  g_encoder_calls++;
  if (rank != 2 || ((uintptr_t)base & 15) || strides[0] % 16 || box[0] == 0 || box[0] > 256 || box[1] == 0 ||
      box[1] > 256 || box[1] != dims[1] || es[0] != 1 || es[1] != 1)
    return CUDA_ERROR_INVALID_VALUE;
  // every fifth call fails as well: the layout must then copy those columns
  // one by one (and may try a shorter run from the next column)
  if (g_encoder_calls % 5 == 0) return CUDA_ERROR_INVALID_VALUE;
  memset(m, 0, sizeof *m);
  return CUDA_SUCCESS;
}

extern "C" void* gb_tensormap_encoder(void) { return (void*)&check_encoder; }
extern "C" int gb_fail(gpu_Context*, const char* fmt, ...)
{
  va_list a;
  va_start(a, fmt);
  vprintf(fmt, a);
  va_end(a);
  printf("\n");
  return -1;
}
extern "C" void* gb_workspace(gpu_Context*, size_t) { return 0; }
extern "C" int gb_cuda_check(gpu_Context*, int, const char*) { return 0; }
extern "C" void gb_prof_begin(gpu_Context*, gb_prof_rec*, int) {}
extern "C" void gb_prof_end(gpu_Context*, gb_prof_rec*, double, double) {}
extern "C" int gb_mv_fill_cols(const gpu_MultiVector*, blk_cols*, int) { return 0; }
extern "C" void* gb_device_alloc(gpu_Context*, size_t) { return 0; }
extern "C" int gb_memcpy_d2h(gpu_Context*, void*, const void*, size_t) { return 0; }
extern "C" int gb_device_error(gpu_Context*, int*) { return 0; }
extern "C" void gb_count_launch(long long) {}
extern "C" void gb_device_free(void*) {}
extern "C" int gb_sync(gpu_Context*) { return 0; }

// the kind of slot j of tile b as the kernel sees it (0 absent, 1 FP32, 2 FP64)
static int slot_kind(const ozg_params& prm, int b, int j, const void** ptr)
{
  if (j < 64) {
    if (j >= prm.h) return 0;
    *ptr = prm.cols.col[j];
    return prm.ldt == GPU_MV_FLOAT64 ? 2 : 1;
  }
  const int q = j - 64;
  if (b >= prm.nq || q >= prm.qw[b]) return 0;
  *ptr = prm.cols.col[64 + 64 * b + q];
  return prm.qdt[b] == GPU_MV_FLOAT64 ? 2 : 1;
}

#define FAIL(...)            \
  do {                       \
    printf(__VA_ARGS__);     \
    printf(" (case %d)\n", it); \
    return 1;                \
  } while (0)

int main(int argc, char** argv)
{
  const int cases = argc > 1 ? atoi(argv[1]) : 100000;
  std::mt19937 rng(12345);
  long tiles = 0, maps = 0;
  static ozg_params prm;
  for (int it = 0; it < cases; it++) {
    memset(&prm, 0, sizeof prm);
    const long n = (it % 7 == 0) ? 1 + (long)(rng() % 300) : 100 + (long)(rng() % 3000000);
    prm.n = n;
    prm.h = 1 + (int)(rng() % 64);
    prm.ldt = rng() % 2 ? GPU_MV_FLOAT64 : GPU_MV_FLOAT32;
    const int ntiles = 1 + (int)(rng() % OZG_MAXQ);
    prm.nq = rng() % 5 == 0 ? 0 : ntiles;
    // a block's columns: 0 contiguous, 1 with masked columns skipped,
    // 2 scattered, 3 contiguous with occasional 16-byte shifts
    auto block = [&](int w, int es, const void** out) {
      const long ld = ((n + 31) / 32) * 32 + 32 * (long)(rng() % 3);
      uintptr_t base = 0x100000000ull + ((uintptr_t)(rng() % 1000000) << 8);
      const int mode = (int)(rng() % 4);
      long c = 0;
      for (int j = 0; j < w; j++) {
        if (mode == 1 && rng() % 5 == 0) c++;
        if (mode == 3 && rng() % 7 == 0) base += 16;
        out[j] = (const void*)(base + (uintptr_t)(c * ld * es) +
                               (mode == 2 ? (uintptr_t)(rng() % 4) * 65536 : 0));
        c++;
      }
    };
    block(prm.h, prm.ldt == GPU_MV_FLOAT64 ? 8 : 4, prm.cols.col);
    for (int t = 0; t < prm.nq; t++) {
      prm.qw[t] = 1 + (int)(rng() % 64);
      prm.qdt[t] = rng() % 2 ? GPU_MV_FLOAT64 : GPU_MV_FLOAT32;
      for (int done = 0; done < prm.qw[t];) {  // merged from up to qw blocks
        const int part = 1 + (int)(rng() % (prm.qw[t] - done));
        block(part, prm.qdt[t] == GPU_MV_FLOAT64 ? 8 : 4, prm.cols.col + 64 + 64 * t + done);
        done += part;
      }
    }
    if (ozg_layout(nullptr, &prm, ntiles)) FAIL("layout refused");
    maps += prm.nmaps;
    for (int m = 0; m < prm.nmaps; m++) {
      if (prm.map_tile[m] < -1 || prm.map_tile[m] >= ntiles) FAIL("map %d: tile %d", m, prm.map_tile[m]);
      if (prm.map_slot[m] < 0 || prm.map_slot[m] >= 128) FAIL("map %d: slot %d", m, prm.map_slot[m]);
      if (prm.map_tile[m] < 0 && prm.map_slot[m] != 0) FAIL("map %d: L map at slot %d", m, prm.map_slot[m]);
      if (prm.map_tile[m] >= 0 && prm.map_slot[m] < 64) FAIL("map %d: Q map at slot %d", m, prm.map_slot[m]);
    }
    for (int t = 0; t < ntiles; t++) {
      std::vector<std::pair<long, long>> spans;
      for (int j = 0; j < 128; j++) {
        const void* ptr = nullptr;
        const int kind = slot_kind(prm, t, j, &ptr);
        if (!kind) continue;
        const long es = kind == 2 ? 8 : 4;
        const long stride = kind == 2 ? OZG_STRIDE64 : OZG_STRIDE32;
        const long off = 16L * prm.roff[t][j];
        if (off + stride > OZG_RAW) FAIL("tile %d slot %d outside the buffer", t, j);
        spans.push_back(std::make_pair(off, off + stride));
        int found = 0;
        for (int m = 0; m < prm.nmaps; m++) {
          if (prm.map_tile[m] >= 0 && prm.map_tile[m] != t) continue;
          const int s0 = prm.map_slot[m];
          const int mf64 = s0 < 64 ? prm.ldt == GPU_MV_FLOAT64 : prm.qdt[t] == GPU_MV_FLOAT64;
          const long mstride = mf64 ? OZG_STRIDE64 : OZG_STRIDE32;
          if (prm.map_bytes[m] <= 0 || prm.map_bytes[m] % mstride) FAIL("map %d: %d bytes", m, prm.map_bytes[m]);
          const int r = prm.map_bytes[m] / (int)mstride;
          if (j < s0 || j >= s0 + r) continue;
          found++;
          if (mstride != stride) FAIL("map %d: dtype of slot %d", m, j);
          if (s0 + r > (s0 < 64 ? prm.h : 64 + prm.qw[t])) FAIL("map %d: run past its block", m);
          const long moff = 16L * prm.roff[t][s0];
          if (moff % 128) FAIL("map %d: tile at %ld not 128-byte aligned", m, moff);
          if (off != moff + (long)(j - s0) * stride) FAIL("map %d: slot %d not at the tile's stride", m, j);
          const int g0 = s0 < 64 ? s0 : 64 + 64 * t + (s0 - 64);
          const long d = (const char*)prm.cols.col[g0 + 1] - (const char*)prm.cols.col[g0];
          if ((const char*)ptr != (const char*)prm.cols.col[g0] + (long)(j - s0) * d)
            FAIL("map %d: slot %d not equally spaced", m, j);
          if (d % 16 || d < n * es) FAIL("map %d: column stride %ld", m, d);
        }
        if (found != (prm.by_map[t][j] ? 1 : 0)) FAIL("tile %d slot %d: %d maps, flag %d", t, j, found, prm.by_map[t][j]);
        if (off % 16) FAIL("tile %d slot %d at %ld", t, j, off);
      }
      std::sort(spans.begin(), spans.end());
      for (size_t i = 1; i < spans.size(); i++)
        if (spans[i].first < spans[i - 1].second) FAIL("tile %d: staged columns overlap", t);
      tiles++;
    }
  }
  if (maps == 0 || g_encoder_calls == 0) {
    printf("no tensor map was made\n");
    return 1;
  }
  printf("ok: %ld tiles, %ld maps\n", tiles, maps);
  return 0;
}
