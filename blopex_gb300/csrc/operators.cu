// operators.cu -- device operators with the reference callback signature
// op(void* data, void* X, void* Y), Y(active) = op(X(active)):
//   CSR SpMM (int32 indices), matrix-free variable-coefficient 7-point (3D)
//   and 5-point (2D) stencils, the shifted 27-point graph Laplacian, and
//   diagonal scaling (Jacobi T = D^{-1}, lumped mass B).
// They replace the serial operators of the reference backend
// (blopex_serial_double/pcg_multi/pcg_multi.c:167-193 MatMultiVec and
// blopex_serial_double/matmultivec/matmultivec.c:11-48).
// FP64 and FP32 multivectors are both accepted; FP32 copies of the
// coefficients are made on first use.  Kernels, one thread per row or cell
// with the x gathers of a warp coalesced along the row index:
//   csr_kernel      CSR, 16 columns per pass over the row (FP64, and FP32
//                   blocks with FP64 arithmetic);
//   csr32_kernel    FP32 CSR: the row's entries in registers, the gathers of
//                   four columns issued ahead of their products;
//   st7_tma_kernel  FP32 7-point: plane tiles staged by TMA into a
//                   shared-memory column ring (st7_ring_kernel: the same
//                   with cp.async copies; st7_kernel: scalar, FP64 and the
//                   unaligned cases);
//   st5_kernel, st27_kernel, diag_kernel;
// plus the inner-CG preconditioner (pcg_apply) and the parameter gradients
// of the adjoint module (grad_*_kernel).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "internal.h"
#include "tc_common.cuh"
#include "blas32.cuh"

enum { OPK_CSR = 1, OPK_ST7 = 2, OPK_ST5 = 3, OPK_ST27 = 4, OPK_DIAG = 5, OPK_PCG = 6 };

struct gpu_Operator {
  int kind;
  gpu_Context* ctx;
  long n;
  long nnz;
  int* rowptr;
  int* colidx;
  double* vals;
  float* vals32;
  int nx, ny, nz;
  double shift;
  double* c[3];   // ST7: cx, cy, cz; ST5: cx, cy
  float* c32[3];
  long clen[3];
  double* w;      // ST27: weights, edge-major [e][cell]
  float* w32;
  double* d;      // DIAG
  float* d32;
  // PCG: `iters` steps of conjugate gradients on `inner` (preconditioned by
  // `prec`, may be NULL) from a zero start; work blocks cached per shape
  gpu_Operator* inner;
  gpu_Operator* prec;
  int iters;
  gpu_MultiVector* work[4];  // r, z, p, q
  gpu_MultiVector* io32[2];  // FP32 copies of an FP64 input / output (mixed mode)
  double* coef;              // 4 x BLK_MAXCOLS device doubles
};

static inline cudaStream_t S(gpu_Context* ctx) { return (cudaStream_t)ctx->stream; }

__constant__ int c_st27_off[13][3] = {
    {1, 0, 0},  {-1, 1, 0}, {0, 1, 0},  {1, 1, 0}, {-1, -1, 1}, {0, -1, 1}, {1, -1, 1},
    {-1, 0, 1}, {0, 0, 1},  {1, 0, 1},  {-1, 1, 1}, {0, 1, 1},  {1, 1, 1}};
static const int h_st27_off[13][3] = {
    {1, 0, 0},  {-1, 1, 0}, {0, 1, 0},  {1, 1, 0}, {-1, -1, 1}, {0, -1, 1}, {1, -1, 1},
    {-1, 0, 1}, {0, 0, 1},  {1, 0, 1},  {-1, 1, 1}, {0, 1, 1},  {1, 1, 1}};

#define OP_CB 16

// ---------------------------------------------------------------- CSR
// T: block element type, V: value type, A: arithmetic (FP64 coefficients
// and accumulation on FP32 blocks when the product must not lose the
// cancellation of a smooth block: see gb_operator_apply)
template <typename T, typename V, typename A = T>
__global__ void __launch_bounds__(256) csr_kernel(long n, const int* __restrict__ rowptr,
                                                  const int* __restrict__ colidx,
                                                  const V* __restrict__ vals, blk_cols X,
                                                  blk_cols Y, int w)
{
  long r = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int p0 = rowptr[r], p1 = rowptr[r + 1];
  for (int c0 = 0; c0 < w; c0 += OP_CB) {
    A acc[OP_CB];
#pragma unroll
    for (int b = 0; b < OP_CB; b++) acc[b] = A(0);
    for (int p = p0; p < p1; p++) {
      const int ci = colidx[p];
      const A v = (A)vals[p];
#pragma unroll
      for (int b = 0; b < OP_CB; b++)
        if (c0 + b < w) acc[b] = fma(v, (A)((const T*)X.col[c0 + b])[ci], acc[b]);
    }
#pragma unroll
    for (int b = 0; b < OP_CB; b++)
      if (c0 + b < w) ((T*)Y.col[c0 + b])[r] = acc[b];
  }
}

// FP32 CSR with rows of at most CSR32_RC entries: the row's (column, value)
// pairs are read once into registers, and the block columns go four at a
// time with the gathers of all four issued before any multiply-add or store
// (the loads of the next columns no longer wait behind the products of the
// previous ones).  Same products, same order per entry as csr_kernel.
// Longer rows take csr_kernel's loop.
#define CSR32_RC 8
#define CSR32_U 4
__global__ void __launch_bounds__(256) csr32_kernel(long n, const int* __restrict__ rowptr,
                                                    const int* __restrict__ colidx,
                                                    const float* __restrict__ vals,
                                                    const __grid_constant__ blk_cols X,
                                                    const __grid_constant__ blk_cols Y, int w)
{
  const long r = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int p0 = rowptr[r], len = rowptr[r + 1] - p0;
  if (len > CSR32_RC) {
    for (int c = 0; c < w; c++) {
      const float* x = (const float*)X.col[c];
      float acc = 0.f;
      for (int p = p0; p < p0 + len; p++) acc = fmaf(vals[p], x[colidx[p]], acc);
      ((float*)Y.col[c])[r] = acc;
    }
    return;
  }
  int ci[CSR32_RC];
  float va[CSR32_RC];
#pragma unroll
  for (int e = 0; e < CSR32_RC; e++) {
    ci[e] = e < len ? colidx[p0 + e] : 0;
    va[e] = e < len ? vals[p0 + e] : 0.f;
  }
  for (int c0 = 0; c0 < w; c0 += CSR32_U) {
    float v[CSR32_U][CSR32_RC];
#pragma unroll
    for (int u = 0; u < CSR32_U; u++) {
      const float* x = (const float*)X.col[c0 + u < w ? c0 + u : c0];
#pragma unroll
      for (int e = 0; e < CSR32_RC; e++) v[u][e] = e < len ? x[ci[e]] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < CSR32_U; u++) {
      if (c0 + u < w) {
        float acc = 0.f;
#pragma unroll
        for (int e = 0; e < CSR32_RC; e++)
          if (e < len) acc = fmaf(va[e], v[u][e], acc);
        ((float*)Y.col[c0 + u])[r] = acc;
      }
    }
  }
}

// ------------------------------------------------------------ 7-point
// One thread per cell, a CTA per 32 x 8 tile of a plane (the y-neighbours
// of the tile's cells are mostly inside the tile: L1 hits; the tiles of the
// neighbouring planes run 1 plane of CTAs earlier / later: L2 hits).  The
// block columns go four at a time: the 28 neighbour loads of four columns
// are issued before any of the four stores (Y may alias X as far as the
// compiler knows, so loads would otherwise wait for the previous column's
// store); the six face coefficients are read once per cell.
#define ST_TX 32
#define ST_TY 8
template <typename T, typename A = T>
__global__ void __launch_bounds__(ST_TX* ST_TY) st7_kernel(int nx, int ny, int nz,
                                                           const A* __restrict__ cx,
                                                           const A* __restrict__ cy,
                                                           const A* __restrict__ cz, A shift,
                                                           blk_cols X, blk_cols Y, int w)
{
  const int tiles_x = (nx + ST_TX - 1) / ST_TX, tiles_y = (ny + ST_TY - 1) / ST_TY;
  const long b = blockIdx.x;
  const int tile = (int)(b % ((long)tiles_x * tiles_y));
  const int k = (int)(b / ((long)tiles_x * tiles_y));
  const int i = (tile % tiles_x) * ST_TX + (int)(threadIdx.x % ST_TX);
  const int j = (tile / tiles_x) * ST_TY + (int)(threadIdx.x / ST_TX);
  if (i >= nx || j >= ny || k >= nz) return;
  const long plane = (long)nx * ny;
  const long c = (long)i + (long)nx * j + plane * k;
  const long jk = (long)j + (long)ny * k;
  const A cw = cx[i + (long)(nx + 1) * jk];
  const A ce = cx[i + 1 + (long)(nx + 1) * jk];
  const A cs = cy[i + (long)nx * (j + (long)(ny + 1) * k)];
  const A cn = cy[i + (long)nx * (j + 1 + (long)(ny + 1) * k)];
  const A cb = cz[c];
  const A ct = cz[c + plane];
  const A dg = cw + ce + cs + cn + cb + ct + shift;
  // neighbour offsets, pointing at the cell itself (weight 0) off the grid
  const long ow = i > 0 ? -1 : 0, oe = i < nx - 1 ? 1 : 0;
  const long os = j > 0 ? -(long)nx : 0, on = j < ny - 1 ? (long)nx : 0;
  const long ob = k > 0 ? -plane : 0, ot = k < nz - 1 ? plane : 0;
  const A ww = i > 0 ? cw : A(0), we = i < nx - 1 ? ce : A(0);
  const A ws = j > 0 ? cs : A(0), wn = j < ny - 1 ? cn : A(0);
  const A wb = k > 0 ? cb : A(0), wt = k < nz - 1 ? ct : A(0);
  constexpr int U = 4;
  for (int col0 = 0; col0 < w; col0 += U) {
    A v[U][7];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const T* x = (const T*)X.col[col0 + u < w ? col0 + u : col0];
      v[u][0] = x[c];
      v[u][1] = x[c + ow];
      v[u][2] = x[c + oe];
      v[u][3] = x[c + os];
      v[u][4] = x[c + on];
      v[u][5] = x[c + ob];
      v[u][6] = x[c + ot];
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      if (col0 + u < w)
        ((T*)Y.col[col0 + u])[c] = (T)(dg * v[u][0] - ww * v[u][1] - we * v[u][2] - ws * v[u][3] -
                                       wn * v[u][4] - wb * v[u][5] - wt * v[u][6]);
    }
  }
}

// ------------------------------------------------- 7-point, FP32 column ring
// FP32 blocks, nx a multiple of 4, 16-byte-aligned input columns.  A CTA owns
// a 32 x 32 tile of one plane (each thread four cells stacked in y) and
// walks the block columns.  Per column it needs the tile with a one-cell
// halo in x and y (34 rows of 40 floats, cells at offsets 4-35) and the tiles
// of the planes below and above: 3408 floats, copied as 784 16-byte pieces
// and 68 4-byte x-halo cells with cp.async (the plan, up to four copies per
// thread, is the same for every column) into a ring of ST7R_DEPTH slots,
// ST7R_DEPTH - 1 columns ahead of the column being computed.  The bytes in
// flight occupy shared memory instead of registers, loads of X never wait
// behind stores of Y, and the y neighbours of a thread's cells come from its
// own registers.  Neighbours off the grid are zero-filled (src-size 0) and
// carry zero weights.  No spin-waits: the ring is ordered by
// cp.async.wait_group and one barrier per column.
#define ST7R_DEPTH 3
#define ST7R_ROW 40
#define ST7R_BELOW (34 * ST7R_ROW)
#define ST7R_ABOVE (ST7R_BELOW + 1024)
#define ST7R_SLOT (ST7R_ABOVE + 1024)
#define ST7R_PIECES 784  // 16-byte pieces per column
#define ST7R_COPIES 852  // + 68 halo cells

static __device__ __forceinline__ void st7r_copy(uint32_t dst, const float* src, int e, int nbytes)
{
  if (e < ST7R_PIECES)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(nbytes)
                 : "memory");
  else if (e < ST7R_COPIES)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(nbytes)
                 : "memory");
}

__global__ void __launch_bounds__(256) st7_ring_kernel(int nx, int ny, int nz,
                                                       const float* __restrict__ cx,
                                                       const float* __restrict__ cy,
                                                       const float* __restrict__ cz, float shift,
                                                       const __grid_constant__ blk_cols X,
                                                       const __grid_constant__ blk_cols Y, int w)
{
  __shared__ __align__(16) float ring[ST7R_DEPTH * ST7R_SLOT];
  const int t = threadIdx.x, tx = t & 31, ty = t >> 5;
  const int tiles_x = (nx + 31) / 32, tiles_y = (ny + 31) / 32;
  const long b = blockIdx.x;
  const int tile = (int)(b % ((long)tiles_x * tiles_y));
  const int k = (int)(b / ((long)tiles_x * tiles_y));
  const int i0 = (tile % tiles_x) * 32, j0 = (tile / tiles_x) * 32;
  const long plane = (long)nx * ny;

  // copy plan: copy e = t + 256 q; source offset from the column base (the
  // columns hold fewer than 2^31 elements), destination float in the slot,
  // byte count (0 = zero fill)
  int src[4], dst[4], nb[4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int e = t + 256 * q;
    bool ok = false;
    long so = 0;
    int d = 0;
    if (e < 272) {  // centre plane, rows j0-1 .. j0+32, eight pieces each
      const int row = e >> 3, x = i0 + 4 * (e & 7), y = j0 - 1 + row;
      ok = y >= 0 && y < ny && x < nx;
      d = row * ST7R_ROW + 4 + 4 * (e & 7);
      so = (long)x + (long)nx * y + plane * k;
    } else if (e < ST7R_PIECES) {  // planes k-1 and k+1, rows j0 .. j0+31
      const int u = e - 272, above = u >> 8, r = (u >> 3) & 31, x = i0 + 4 * (u & 7), y = j0 + r;
      const int z = above ? k + 1 : k - 1;
      ok = y < ny && x < nx && z >= 0 && z < nz;
      d = (above ? ST7R_ABOVE : ST7R_BELOW) + r * 32 + 4 * (u & 7);
      so = (long)x + (long)nx * y + plane * z;
    } else if (e < ST7R_COPIES) {  // x halo: cells i0-1 and i0+32 of the 34 centre rows
      const int u = e - ST7R_PIECES, row = u >> 1, east = u & 1;
      const int x = east ? i0 + 32 : i0 - 1, y = j0 - 1 + row;
      ok = y >= 0 && y < ny && x >= 0 && x < nx;
      d = row * ST7R_ROW + (east ? 36 : 3);
      so = (long)x + (long)nx * y + plane * k;
    }
    src[q] = ok ? (int)so : 0;
    dst[q] = d;
    nb[q] = ok ? (e < ST7R_PIECES ? 16 : 4) : 0;
  }
  const uint32_t ring_s = (uint32_t)__cvta_generic_to_shared(ring);

#pragma unroll 1
  for (int c = 0; c < ST7R_DEPTH - 1; c++) {
    if (c < w) {
      const float* base = (const float*)X.col[c];
#pragma unroll
      for (int q = 0; q < 4; q++)
        st7r_copy(ring_s + 4u * (ST7R_SLOT * c + dst[q]), base + src[q], t + 256 * q, nb[q]);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  }

  // coefficients of the thread's four cells (rows j0 + 4 ty .. + 3)
  const int i = i0 + tx, jb = j0 + 4 * ty;
  float dg[4], ww[4], we[4], ws[4], wn[4], wb[4], wt[4];
  bool valid[4];
#pragma unroll
  for (int s = 0; s < 4; s++) {
    const int j = jb + s;
    valid[s] = i < nx && j < ny;
    dg[s] = ww[s] = we[s] = ws[s] = wn[s] = wb[s] = wt[s] = 0.f;
    if (valid[s]) {
      const long cell = (long)i + (long)nx * j + plane * k;
      const long jk = (long)j + (long)ny * k;
      const float cw = cx[i + (long)(nx + 1) * jk];
      const float ce = cx[i + 1 + (long)(nx + 1) * jk];
      const float cs = cy[i + (long)nx * (j + (long)(ny + 1) * k)];
      const float cn = cy[i + (long)nx * (j + 1 + (long)(ny + 1) * k)];
      const float cb = cz[cell];
      const float ct = cz[cell + plane];
      dg[s] = cw + ce + cs + cn + cb + ct + shift;
      ww[s] = i > 0 ? cw : 0.f;
      we[s] = i < nx - 1 ? ce : 0.f;
      ws[s] = j > 0 ? cs : 0.f;
      wn[s] = j < ny - 1 ? cn : 0.f;
      wb[s] = k > 0 ? cb : 0.f;
      wt[s] = k < nz - 1 ? ct : 0.f;
    }
  }
  const long cell0 = (long)i + (long)nx * jb + plane * k;

  int slot = 0, ahead_slot = ST7R_DEPTH - 1;
#pragma unroll 1
  for (int col = 0; col < w; col++) {
    asm volatile("cp.async.wait_group %0;" ::"n"(ST7R_DEPTH - 2) : "memory");
    __syncthreads();  // column col landed for all threads; the slot of col - 1 is free
    const int ahead = col + ST7R_DEPTH - 1;
    if (ahead < w) {
      const float* base = (const float*)X.col[ahead];
      const uint32_t so = ring_s + 4u * ST7R_SLOT * ahead_slot;
#pragma unroll
      for (int q = 0; q < 4; q++) st7r_copy(so + 4u * dst[q], base + src[q], t + 256 * q, nb[q]);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    const float* sl = ring + ST7R_SLOT * slot;
    float cv[6];
#pragma unroll
    for (int r = 0; r < 6; r++) cv[r] = sl[(4 * ty + r) * ST7R_ROW + 4 + tx];
    float* y = (float*)Y.col[col] + cell0;
#pragma unroll
    for (int s = 0; s < 4; s++) {
      const int m = (4 * ty + 1 + s) * ST7R_ROW + 4 + tx;
      const float v1 = sl[m - 1], v2 = sl[m + 1];
      const float v5 = sl[ST7R_BELOW + (4 * ty + s) * 32 + tx];
      const float v6 = sl[ST7R_ABOVE + (4 * ty + s) * 32 + tx];
      if (valid[s])
        __stcs(y + (long)nx * s, dg[s] * cv[s + 1] - ww[s] * v1 - we[s] * v2 - ws[s] * cv[s] -
                                     wn[s] * cv[s + 2] - wb[s] * v5 - wt[s] * v6);
    }
    slot = slot == ST7R_DEPTH - 1 ? 0 : slot + 1;
    ahead_slot = ahead_slot == ST7R_DEPTH - 1 ? 0 : ahead_slot + 1;
  }
}

// ------------------------------------------- 7-point, FP32, TMA column ring
// The column ring of st7_ring_kernel with the copies done by the tensor
// memory accelerator: per column one thread issues three 4D tensor loads
// (x, y, z, block column) on one mbarrier -- the 40 x 34 centre box from
// (i0 - 4, j0 - 1, k) and the 32 x 32 boxes of planes k - 1 and k + 1 --
// and TMA writes the same shared-memory layout the cp.async plan builds
// (centre rows of 40 floats, cells at offsets 4-35), filling everything off
// the grid with zeros.  x coordinates are multiples of 4 floats (16 bytes);
// every box starts on a 128-byte boundary of its slot.  Waits are bounded: a
// timeout stops the issue of further copies, poisons the CTA's outputs with
// NaN, sets the context's device error word and, before the CTA exits,
// waits (bounded again) for the copies still in flight.
#define ST7T_DEPTH 3
#define ST7T_BELOW 1376  // floats: the 34 x 40 centre box, padded to 128 bytes
#define ST7T_ABOVE (ST7T_BELOW + 1024)
#define ST7T_SLOT (ST7T_ABOVE + 1024)            // 13696 bytes, a multiple of 128
#define ST7T_BYTES ((34 * 40 + 2 * 32 * 32) * 4)  // bytes per column (13632)

struct st7t_cols {
  int c[BLK_MAXCOLS];  // physical column of each active column
};

static __device__ __forceinline__ void st7t_load(uint32_t dst, const CUtensorMap* map, int x, int y,
                                                 int z, int c, uint32_t bar)
{
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
      "%3, %4, %5}], [%6];" ::"r"(dst),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(c), "r"(bar)
      : "memory");
}

__global__ void __launch_bounds__(256) st7_tma_kernel(
    int nx, int ny, int nz, const float* __restrict__ cx, const float* __restrict__ cy,
    const float* __restrict__ cz, float shift, const __grid_constant__ CUtensorMap tm_c,
    const __grid_constant__ CUtensorMap tm_z, const __grid_constant__ st7t_cols XC,
    const __grid_constant__ blk_cols Y, int w, int* err, double* __restrict__ dotp)
{
  __shared__ __align__(128) float ring[ST7T_DEPTH * ST7T_SLOT];
  __shared__ __align__(8) uint64_t bar[ST7T_DEPTH];
  __shared__ int abort_flag;
  const int t = threadIdx.x, tx = t & 31, ty = t >> 5;
  const int tiles_x = (nx + 31) / 32, tiles_y = (ny + 31) / 32;
  const long b = blockIdx.x;
  const int tile = (int)(b % ((long)tiles_x * tiles_y));
  const int k = (int)(b / ((long)tiles_x * tiles_y));
  const int i0 = (tile % tiles_x) * 32, j0 = (tile / tiles_x) * 32;
  const long plane = (long)nx * ny;
  if (t == 0) {
    abort_flag = 0;
    for (int q = 0; q < ST7T_DEPTH; q++) mbar_init(&bar[q], 1);
  }
  fence_proxy_async();
  __syncthreads();
  const uint32_t ring_s = smem_u32(ring);
  int issued = 0, waited = 0;  // thread 0: columns issued / columns whose copies it saw land
  if (t == 0) {
    for (int c = 0; c < ST7T_DEPTH - 1 && c < w; c++) {
      const uint32_t bq = smem_u32(&bar[c]), d = ring_s + 4u * ST7T_SLOT * c;
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bq),
                   "r"((uint32_t)ST7T_BYTES)
                   : "memory");
      st7t_load(d, &tm_c, i0 - 4, j0 - 1, k, XC.c[c], bq);
      st7t_load(d + 4u * ST7T_BELOW, &tm_z, i0, j0, k - 1, XC.c[c], bq);
      st7t_load(d + 4u * ST7T_ABOVE, &tm_z, i0, j0, k + 1, XC.c[c], bq);
      issued++;
    }
  }

  // coefficients of the thread's four cells (rows j0 + 4 ty .. + 3)
  const int i = i0 + tx, jb = j0 + 4 * ty;
  float dg[4], ww[4], we[4], ws[4], wn[4], wb[4], wt[4];
  bool valid[4];
#pragma unroll
  for (int s = 0; s < 4; s++) {
    const int j = jb + s;
    valid[s] = i < nx && j < ny;
    dg[s] = ww[s] = we[s] = ws[s] = wn[s] = wb[s] = wt[s] = 0.f;
    if (valid[s]) {
      const long cell = (long)i + (long)nx * j + plane * k;
      const long jk = (long)j + (long)ny * k;
      const float cw = cx[i + (long)(nx + 1) * jk];
      const float ce = cx[i + 1 + (long)(nx + 1) * jk];
      const float cs = cy[i + (long)nx * (j + (long)(ny + 1) * k)];
      const float cn = cy[i + (long)nx * (j + 1 + (long)(ny + 1) * k)];
      const float cb = cz[cell];
      const float ct = cz[cell + plane];
      dg[s] = cw + ce + cs + cn + cb + ct + shift;
      ww[s] = i > 0 ? cw : 0.f;
      we[s] = i < nx - 1 ? ce : 0.f;
      ws[s] = j > 0 ? cs : 0.f;
      wn[s] = j < ny - 1 ? cn : 0.f;
      wb[s] = k > 0 ? cb : 0.f;
      wt[s] = k < nz - 1 ? ct : 0.f;
    }
  }
  const long cell0 = (long)i + (long)nx * jb + plane * k;

  int slot = 0, ahead_slot = ST7T_DEPTH - 1;
#pragma unroll 1
  for (int col = 0; col < w; col++) {
    const uint32_t parity = (uint32_t)((col / ST7T_DEPTH) & 1);
    const bool ok = !abort_flag && mbar_wait(&bar[slot], parity, &abort_flag);
    if (!ok) abort_flag = 1;
    else if (t == 0) waited = col + 1;
    __syncthreads();  // column col landed; every thread is done with the slot of col - 1
    const bool go = !abort_flag;
    const int ahead = col + ST7T_DEPTH - 1;
    if (go && t == 0 && ahead < w) {
      const uint32_t bq = smem_u32(&bar[ahead_slot]), d = ring_s + 4u * ST7T_SLOT * ahead_slot;
      fence_proxy_async();
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bq),
                   "r"((uint32_t)ST7T_BYTES)
                   : "memory");
      st7t_load(d, &tm_c, i0 - 4, j0 - 1, k, XC.c[ahead], bq);
      st7t_load(d + 4u * ST7T_BELOW, &tm_z, i0, j0, k - 1, XC.c[ahead], bq);
      st7t_load(d + 4u * ST7T_ABOVE, &tm_z, i0, j0, k + 1, XC.c[ahead], bq);
      issued++;
    }
    float* y = (float*)Y.col[col] + cell0;
    float xs = 0.f, xc = 0.f;  // this thread's share of x' (A x): compensated sum
    if (go) {
      const float* sl = ring + ST7T_SLOT * slot;
      float cv[6];
#pragma unroll
      for (int r = 0; r < 6; r++) cv[r] = sl[(4 * ty + r) * 40 + 4 + tx];
#pragma unroll
      for (int s = 0; s < 4; s++) {
        const int m = (4 * ty + 1 + s) * 40 + 4 + tx;
        const float v1 = sl[m - 1], v2 = sl[m + 1];
        const float v5 = sl[ST7T_BELOW + (4 * ty + s) * 32 + tx];
        const float v6 = sl[ST7T_ABOVE + (4 * ty + s) * 32 + tx];
        if (valid[s]) {
          const float yv = dg[s] * cv[s + 1] - ww[s] * v1 - we[s] * v2 - ws[s] * cv[s] -
                           wn[s] * cv[s + 2] - wb[s] * v5 - wt[s] * v6;
          __stcs(y + (long)nx * s, yv);
          if (dotp) acc_prod32(xs, xc, cv[s + 1], yv);
        }
      }
    }
    if (dotp) {
      // per warp: exact products in compensated FP32 sums, combined across
      // the lanes by two-sums, into FP64 partials that a second kernel sums
      // in a fixed order (the inner CG's p' A p, as accurate as its
      // separate inner-product kernel)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float s2 = __shfl_xor_sync(0xffffffffu, xs, o);
        const float c2 = __shfl_xor_sync(0xffffffffu, xc, o);
        const float t2 = __fadd_rn(xs, s2);
        const float bp = __fsub_rn(t2, xs);
        const float e = __fadd_rn(__fsub_rn(xs, __fsub_rn(t2, bp)), __fsub_rn(s2, bp));
        xs = t2;
        xc = __fadd_rn(__fadd_rn(xc, c2), e);
      }
      if (tx == 0) dotp[(long)col * gridDim.x * 8 + blockIdx.x * 8 + ty] = go ? (double)xs + (double)xc : 0.0;
    }
    if (!go) {
#pragma unroll
      for (int s = 0; s < 4; s++)
        if (valid[s]) y[(long)nx * s] = __int_as_float(0x7fc00000);  // NaN: output incomplete
    }
    slot = slot == ST7T_DEPTH - 1 ? 0 : slot + 1;
    ahead_slot = ahead_slot == ST7T_DEPTH - 1 ? 0 : ahead_slot + 1;
  }
  if (t == 0 && abort_flag) {
    atomicExch(err, 1);
    // copies issued but not seen landing: wait for them before the CTA exits
    for (int c = waited; c < issued; c++)
      mbar_drain(&bar[c % ST7T_DEPTH], (uint32_t)((c / ST7T_DEPTH) & 1));
  }
}

// ------------------------------------------------------------ 5-point
template <typename T>
__global__ void __launch_bounds__(256) st5_kernel(int nx, int ny, const T* __restrict__ cx,
                                                  const T* __restrict__ cy, T shift, blk_cols X,
                                                  blk_cols Y, int w)
{
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  long n = (long)nx * ny;
  if (c >= n) return;
  const int i = (int)(c % nx);
  const int j = (int)(c / nx);
  const T cw = cx[i + (long)(nx + 1) * j];
  const T ce = cx[i + 1 + (long)(nx + 1) * j];
  const T cs = cy[c];
  const T cn = cy[c + nx];
  const T dg = cw + ce + cs + cn + shift;
  for (int col = 0; col < w; col++) {
    const T* x = (const T*)X.col[col];
    T v = dg * x[c];
    if (i > 0) v -= cw * x[c - 1];
    if (i < nx - 1) v -= ce * x[c + 1];
    if (j > 0) v -= cs * x[c - nx];
    if (j < ny - 1) v -= cn * x[c + nx];
    ((T*)Y.col[col])[c] = v;
  }
}

// ----------------------------------------------------------- 27-point
// weights stored edge-major: w[e*n + cell] for the forward edge e of cell
template <typename T>
__global__ void __launch_bounds__(256) st27_kernel(int nx, int ny, int nz, const T* __restrict__ wt,
                                                   T shift, blk_cols X, blk_cols Y, int w)
{
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long n = (long)nx * ny * nz;
  if (c >= n) return;
  const int i = (int)(c % nx);
  const int j = (int)((c / nx) % ny);
  const int k = (int)(c / ((long)nx * ny));
  T we[26];
  long nb[26];
  T dg = shift;
#pragma unroll
  for (int e = 0; e < 13; e++) {
    // forward edge (c, c + off_e) and backward edge (c - off_e, c)
    const int di = c_st27_off[e][0], dj = c_st27_off[e][1], dk = c_st27_off[e][2];
    const int i2 = i + di, j2 = j + dj, k2 = k + dk;
    const long off = di + (long)nx * (dj + (long)ny * dk);
    if (i2 >= 0 && i2 < nx && j2 >= 0 && j2 < ny && k2 >= 0 && k2 < nz) {
      we[e] = wt[e * n + c];
      nb[e] = c + off;
    } else {
      we[e] = T(0);
      nb[e] = c;
    }
    const int i3 = i - di, j3 = j - dj, k3 = k - dk;
    if (i3 >= 0 && i3 < nx && j3 >= 0 && j3 < ny && k3 >= 0 && k3 < nz) {
      we[13 + e] = wt[e * n + c - off];
      nb[13 + e] = c - off;
    } else {
      we[13 + e] = T(0);
      nb[13 + e] = c;
    }
    dg += we[e] + we[13 + e];
  }
  for (int col = 0; col < w; col++) {
    const T* x = (const T*)X.col[col];
    T v = dg * x[c];
#pragma unroll
    for (int e = 0; e < 26; e++) v -= we[e] * x[nb[e]];
    ((T*)Y.col[col])[c] = v;
  }
}

// ----------------------------------------------------------- diagonal
template <typename T, typename V>
__global__ void diag_kernel(long n, const V* __restrict__ d, blk_cols X, blk_cols Y)
{
  const T* x = (const T*)X.col[blockIdx.y];
  T* y = (T*)Y.col[blockIdx.y];
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
    y[r] = (T)d[r] * x[r];
}

// ------------------------------------------------------------ helpers
template <typename TI, typename TO>
__global__ void cast_kernel(const TI* __restrict__ a, TO* __restrict__ b, long n)
{
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
    b[r] = (TO)a[r];
}

static float* make_f32(gpu_Context* ctx, const double* src, long n)
{
  float* dst = (float*)gb_device_alloc(ctx, sizeof(float) * (size_t)(n > 0 ? n : 1));
  if (!dst) return NULL;
  unsigned blocks = (unsigned)((n + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  if (blocks < 1) blocks = 1;
  cast_kernel<double, float><<<blocks, 256, 0, S(ctx)>>>(src, dst, n);
  gb_count_launch(1);
  if (gb_cuda_check(ctx, (int)cudaGetLastError(), "cast")) {
    gb_device_free(dst);
    return NULL;
  }
  return dst;
}

static double* upload(gpu_Context* ctx, const void* host, size_t bytes)
{
  double* d = (double*)gb_device_alloc(ctx, bytes);
  if (!d) return NULL;
  if (gb_memcpy_h2d(ctx, d, host, bytes)) {
    gb_device_free(d);
    return NULL;
  }
  return d;
}

static gpu_Operator* op_new(gpu_Context* ctx, int kind, long n)
{
  gpu_Operator* op = (gpu_Operator*)calloc(1, sizeof(gpu_Operator));
  op->kind = kind;
  op->ctx = ctx;
  op->n = n;
  return op;
}

extern "C" void gpu_OperatorDestroy(gpu_Operator* op)
{
  if (!op) return;
  cudaStreamSynchronize(S(op->ctx));
  gb_device_free(op->rowptr);
  gb_device_free(op->colidx);
  gb_device_free(op->vals);
  gb_device_free(op->vals32);
  for (int a = 0; a < 3; a++) {
    gb_device_free(op->c[a]);
    gb_device_free(op->c32[a]);
  }
  gb_device_free(op->w);
  gb_device_free(op->w32);
  gb_device_free(op->d);
  gb_device_free(op->d32);
  for (int b = 0; b < 4; b++) gpu_MultiVectorDestroy(op->work[b]);
  for (int b = 0; b < 2; b++) gpu_MultiVectorDestroy(op->io32[b]);
  gb_device_free(op->coef);
  free(op);
}

extern "C" gpu_Operator* gpu_CSRMatrixCreate(gpu_Context* ctx, long n, long nnz, const int* rowptr,
                                             const int* colidx, const double* vals)
{
  if (n <= 0 || nnz < 0) {
    gb_fail(ctx, "CSR: bad sizes n=%ld nnz=%ld", n, nnz);
    return NULL;
  }
  gpu_Operator* op = op_new(ctx, OPK_CSR, n);
  op->nnz = nnz;
  op->rowptr = (int*)upload(ctx, rowptr, sizeof(int) * (size_t)(n + 1));
  op->colidx = (int*)upload(ctx, colidx, sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
  op->vals = upload(ctx, vals, sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
  if (!op->rowptr || !op->colidx || !op->vals) {
    gpu_OperatorDestroy(op);
    return NULL;
  }
  return op;
}

extern "C" gpu_Operator* gpu_Stencil7Create(gpu_Context* ctx, int nx, int ny, int nz,
                                            const double* cx, const double* cy, const double* cz,
                                            double shift)
{
  if (nx <= 0 || ny <= 0 || nz <= 0) {
    gb_fail(ctx, "stencil7: bad grid %d x %d x %d", nx, ny, nz);
    return NULL;
  }
  gpu_Operator* op = op_new(ctx, OPK_ST7, (long)nx * ny * nz);
  op->nx = nx;
  op->ny = ny;
  op->nz = nz;
  op->shift = shift;
  op->clen[0] = (long)(nx + 1) * ny * nz;
  op->clen[1] = (long)nx * (ny + 1) * nz;
  op->clen[2] = (long)nx * ny * (nz + 1);
  const double* src[3] = {cx, cy, cz};
  for (int a = 0; a < 3; a++) {
    op->c[a] = upload(ctx, src[a], sizeof(double) * (size_t)op->clen[a]);
    if (!op->c[a]) {
      gpu_OperatorDestroy(op);
      return NULL;
    }
  }
  return op;
}

extern "C" gpu_Operator* gpu_Stencil5Create(gpu_Context* ctx, int nx, int ny, const double* cx,
                                            const double* cy, double shift)
{
  if (nx <= 0 || ny <= 0) {
    gb_fail(ctx, "stencil5: bad grid %d x %d", nx, ny);
    return NULL;
  }
  gpu_Operator* op = op_new(ctx, OPK_ST5, (long)nx * ny);
  op->nx = nx;
  op->ny = ny;
  op->nz = 1;
  op->shift = shift;
  op->clen[0] = (long)(nx + 1) * ny;
  op->clen[1] = (long)nx * (ny + 1);
  const double* src[2] = {cx, cy};
  for (int a = 0; a < 2; a++) {
    op->c[a] = upload(ctx, src[a], sizeof(double) * (size_t)op->clen[a]);
    if (!op->c[a]) {
      gpu_OperatorDestroy(op);
      return NULL;
    }
  }
  return op;
}

extern "C" gpu_Operator* gpu_Stencil27Create(gpu_Context* ctx, int nx, int ny, int nz,
                                             const double* w, double shift)
{
  if (nx <= 0 || ny <= 0 || nz <= 0) {
    gb_fail(ctx, "stencil27: bad grid %d x %d x %d", nx, ny, nz);
    return NULL;
  }
  long n = (long)nx * ny * nz;
  gpu_Operator* op = op_new(ctx, OPK_ST27, n);
  op->nx = nx;
  op->ny = ny;
  op->nz = nz;
  op->shift = shift;
  // re-lay the caller's cell-major weights edge-major for coalesced reads
  double* tmp = (double*)malloc(sizeof(double) * (size_t)n * 13);
  if (!tmp) {
    gb_fail(ctx, "stencil27: host allocation failed");
    free(op);
    return NULL;
  }
  for (long c = 0; c < n; c++)
    for (int e = 0; e < 13; e++) tmp[(size_t)e * n + c] = w[13 * c + e];
  op->w = upload(ctx, tmp, sizeof(double) * (size_t)n * 13);
  free(tmp);
  if (!op->w) {
    gpu_OperatorDestroy(op);
    return NULL;
  }
  return op;
}

extern "C" gpu_Operator* gpu_DiagonalCreate(gpu_Context* ctx, long n, const double* d)
{
  if (n <= 0) {
    gb_fail(ctx, "diagonal: bad size %ld", n);
    return NULL;
  }
  gpu_Operator* op = op_new(ctx, OPK_DIAG, n);
  op->d = upload(ctx, d, sizeof(double) * (size_t)n);
  if (!op->d) {
    gpu_OperatorDestroy(op);
    return NULL;
  }
  return op;
}

static int ensure_f32(gpu_Operator* op)
{
  gpu_Context* ctx = op->ctx;
  switch (op->kind) {
    case OPK_CSR:
      if (!op->vals32 && !(op->vals32 = make_f32(ctx, op->vals, op->nnz))) return -1;
      break;
    case OPK_ST7:
    case OPK_ST5:
      for (int a = 0; a < (op->kind == OPK_ST7 ? 3 : 2); a++)
        if (!op->c32[a] && !(op->c32[a] = make_f32(ctx, op->c[a], op->clen[a]))) return -1;
      break;
    case OPK_ST27:
      if (!op->w32 && !(op->w32 = make_f32(ctx, op->w, op->n * 13))) return -1;
      break;
    case OPK_DIAG:
      if (!op->d32 && !(op->d32 = make_f32(ctx, op->d, op->n))) return -1;
      break;
  }
  return 0;
}

// the ring kernel copies 16-byte pieces (rows of whole 16-byte groups, input
// columns on 16-byte boundaries) and addresses a column with 32-bit offsets
static int st7_ring_ok(const gpu_Operator* op, const blk_cols* xc, int w)
{
  if (op->nx % 4 || op->n >= (1L << 31)) return 0;
  for (int c = 0; c < w; c++)
    if ((uintptr_t)xc->col[c] & 15) return 0;
  return 1;
}

// the tensor-map encoder of the driver (cuTensorMapEncodeTiled), found once
// through the runtime (a function-local static: initialised once, also when
// several host threads ask first); NULL when the driver has none
extern "C" void* gb_tensormap_encoder(void)
{
  static void* const fn = [] {
    void* p = NULL;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = NULL;
    return p;
  }();
  return fn;
}

static PFN_cuTensorMapEncodeTiled_v12000 st7t_encoder(void)
{
  return (PFN_cuTensorMapEncodeTiled_v12000)gb_tensormap_encoder();
}

// tensor maps of the FP32 block X as (x, y, z, column) for st7_tma_kernel:
// boxes 40 x 34 (centre plane with halo) and 32 x 32 (planes above and
// below).  TMA needs 16-byte-aligned bases and strides: nx a multiple of 4
// and ld * 4 a multiple of 16.  Returns 0 when both maps were encoded.
static int st7t_maps(const gpu_Operator* op, const gpu_MultiVector* X, CUtensorMap* mc,
                     CUtensorMap* mz)
{
  PFN_cuTensorMapEncodeTiled_v12000 enc = st7t_encoder();
  if (!enc || op->nx % 4 || ((uintptr_t)X->data & 15) || (X->ld * 4) % 16) return -1;
  const cuuint64_t dims[4] = {(cuuint64_t)op->nx, (cuuint64_t)op->ny, (cuuint64_t)op->nz,
                              (cuuint64_t)X->num_vectors};
  const cuuint64_t strides[3] = {(cuuint64_t)op->nx * 4, (cuuint64_t)op->nx * op->ny * 4,
                                 (cuuint64_t)X->ld * 4};
  const cuuint32_t boxc[4] = {40, 34, 1, 1}, boxz[4] = {32, 32, 1, 1}, es[4] = {1, 1, 1, 1};
  if (enc(mc, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, X->data, dims, strides, boxc, es,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return -1;
  if (enc(mz, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, X->data, dims, strides, boxz, es,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return -1;
  return 0;
}

static int pcg_apply(gpu_Operator* op, gpu_MultiVector* X, gpu_MultiVector* Y);

// the per-column sums of the stencil kernel's warp partials, in a fixed order
__global__ void __launch_bounds__(256) st7t_dot_reduce_kernel(const double* __restrict__ parts,
                                                              long nparts, double* __restrict__ out)
{
  const double* p = parts + (size_t)blockIdx.x * nparts;
  double acc = 0.0;
  for (long i = threadIdx.x; i < nparts; i += blockDim.x) acc += p[i];
  const double t = block_sum256(acc);
  if (threadIdx.x == 0) out[blockIdx.x] = t;
}

static int operator_apply(gpu_Operator* op, gpu_MultiVector* X, gpu_MultiVector* Y, double* dot_out);

extern "C" int gb_operator_apply(gpu_Operator* op, gpu_MultiVector* X, gpu_MultiVector* Y)
{
  return operator_apply(op, X, Y, NULL);
}

// Y = A X and out[c] = X_c' Y_c in one pass where the operator's kernel can
// fold the inner products in (the FP32 TMA 7-point stencil): 0; 1 when it
// cannot (nothing done: apply and take the inner products apart); -1 on error
extern "C" int gb_operator_apply_dot(gpu_Operator* op, gpu_MultiVector* X, gpu_MultiVector* Y,
                                     double* dot_out)
{
  return operator_apply(op, X, Y, dot_out);
}

static int operator_apply(gpu_Operator* op, gpu_MultiVector* X, gpu_MultiVector* Y, double* dot_out)
{
  if (op->kind == OPK_PCG) return dot_out ? 1 : pcg_apply(op, X, Y);
  gpu_Context* ctx = op->ctx;
  if (X->size != op->n || Y->size != op->n)
    return gb_fail(ctx, "operator of size %ld applied to blocks of %ld / %ld rows", op->n,
                   X->size, Y->size);
  if (X->num_active != Y->num_active)
    return gb_fail(ctx, "operator: %d active input columns but %d output columns",
                   X->num_active, Y->num_active);
  if (X->dtype != Y->dtype) return gb_fail(ctx, "operator: mixed dtypes");
  const int w = X->num_active;
  if (w == 0) return 0;
  if (w > BLK_MAXCOLS)
    return gb_fail(ctx, "operator: %d active columns exceed the supported %d", w, BLK_MAXCOLS);
  blk_cols xc, yc;
  gb_mv_fill_cols(X, &xc, 0);
  gb_mv_fill_cols(Y, &yc, 0);
  const int f32 = X->dtype == GPU_MV_FLOAT32;
  if (f32 && ensure_f32(op)) return -1;
  // FP32 blocks, FP64 coefficients and arithmetic (CSR, 7-point): for a
  // smooth block |A x| << |A| |x|, and FP32 products and sums would lose the
  // cancellation that A x consists of
  const int acc64 = f32 && ctx->op_accurate && (op->kind == OPK_CSR || op->kind == OPK_ST7);
  // the FP32 7-point stencil staged by TMA (nx a multiple of 4, aligned block)
  CUtensorMap tmc, tmz;
  const int tma = op->kind == OPK_ST7 && f32 && !acc64 && st7t_maps(op, X, &tmc, &tmz) == 0;
  if (dot_out && !tma) return 1;
  const unsigned st7t_ctas = (unsigned)(((op->nx + 31) / 32) * ((op->ny + 31) / 32) * (long)op->nz);
  double* dparts = NULL;
  if (dot_out && !(dparts = (double*)gb_workspace(ctx, sizeof(double) * 8 * (size_t)st7t_ctas * w)))
    return -1;
  const long n = op->n;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  const double es = f32 ? 4.0 : 8.0;
  double bytes = 2.0 * es * n * w, flops = 0.0;
  int cls = GB_K_DIAG;
  switch (op->kind) {
    case OPK_CSR:
      cls = GB_K_CSR;
      bytes += op->nnz * (es + 4.0) + 4.0 * (n + 1);
      flops = 2.0 * op->nnz * w;
      break;
    case OPK_ST7:
      cls = GB_K_ST7;
      bytes += es * (op->clen[0] + op->clen[1] + op->clen[2]);
      flops = 13.0 * n * w;
      break;
    case OPK_ST5:
      cls = GB_K_ST5;
      bytes += es * (op->clen[0] + op->clen[1]);
      flops = 9.0 * n * w;
      break;
    case OPK_ST27:
      cls = GB_K_ST27;
      bytes += es * 13.0 * n;
      flops = 53.0 * n * w;
      break;
    default:
      bytes += es * n;
      flops = 1.0 * n * w;
  }
  if (f32 && !acc64) {  // FP32 arithmetic: timed apart from the FP64 launches
    switch (cls) {
      case GB_K_CSR: cls = GB_K_CSR32; break;
      case GB_K_ST7: cls = GB_K_ST7_32; break;
      case GB_K_ST5: cls = GB_K_ST5_32; break;
      case GB_K_ST27: cls = GB_K_ST27_32; break;
      default: cls = GB_K_DIAG32;
    }
  }
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, cls);
  switch (op->kind) {
    case OPK_CSR:
      if (acc64)
        csr_kernel<float, double, double><<<blocks, 256, 0, S(ctx)>>>(n, op->rowptr, op->colidx,
                                                                      op->vals, xc, yc, w);
      else if (f32)
        csr32_kernel<<<blocks, 256, 0, S(ctx)>>>(n, op->rowptr, op->colidx, op->vals32, xc, yc, w);
      else
        csr_kernel<double, double><<<blocks, 256, 0, S(ctx)>>>(n, op->rowptr, op->colidx,
                                                               op->vals, xc, yc, w);
      break;
    case OPK_ST7: {
      const unsigned tb = (unsigned)(((op->nx + ST_TX - 1) / ST_TX) * ((op->ny + ST_TY - 1) / ST_TY) *
                                     (long)op->nz);
      if (acc64)
        st7_kernel<float, double><<<tb, ST_TX * ST_TY, 0, S(ctx)>>>(op->nx, op->ny, op->nz, op->c[0],
                                                                    op->c[1], op->c[2], op->shift,
                                                                    xc, yc, w);
      else if (tma) {
        st7t_cols pc;
        for (int c = 0; c < w; c++) pc.c[c] = X->active[c];
        if (tc_apply_wait_polls(ctx->opt.wait_polls, S(ctx)) != cudaSuccess)
          return gb_fail(ctx, "stencil7: cannot set the wait limit");
        st7_tma_kernel<<<st7t_ctas, 256, 0, S(ctx)>>>(op->nx, op->ny, op->nz, op->c32[0], op->c32[1],
                                                      op->c32[2], (float)op->shift, tmc, tmz, pc, yc,
                                                      w, ctx->dcount + 5, dparts);
        if (dot_out) {
          st7t_dot_reduce_kernel<<<w, 256, 0, S(ctx)>>>(dparts, 8L * st7t_ctas, dot_out);
          gb_count_launch(1);
        }
      } else if (f32 && st7_ring_ok(op, &xc, w))
        st7_ring_kernel<<<(unsigned)(((op->nx + 31) / 32) * ((op->ny + 31) / 32) * (long)op->nz), 256,
                          0, S(ctx)>>>(op->nx, op->ny, op->nz, op->c32[0], op->c32[1],
                                                op->c32[2], (float)op->shift, xc, yc, w);
      else if (f32)
        st7_kernel<float><<<tb, ST_TX * ST_TY, 0, S(ctx)>>>(op->nx, op->ny, op->nz, op->c32[0],
                                                            op->c32[1], op->c32[2], (float)op->shift,
                                                            xc, yc, w);
      else
        st7_kernel<double><<<tb, ST_TX * ST_TY, 0, S(ctx)>>>(op->nx, op->ny, op->nz, op->c[0],
                                                             op->c[1], op->c[2], op->shift, xc, yc, w);
    }
      break;
    case OPK_ST5:
      if (f32)
        st5_kernel<float><<<blocks, 256, 0, S(ctx)>>>(op->nx, op->ny, op->c32[0], op->c32[1],
                                                      (float)op->shift, xc, yc, w);
      else
        st5_kernel<double><<<blocks, 256, 0, S(ctx)>>>(op->nx, op->ny, op->c[0], op->c[1],
                                                       op->shift, xc, yc, w);
      break;
    case OPK_ST27:
      if (f32)
        st27_kernel<float><<<blocks, 256, 0, S(ctx)>>>(op->nx, op->ny, op->nz, op->w32,
                                                       (float)op->shift, xc, yc, w);
      else
        st27_kernel<double><<<blocks, 256, 0, S(ctx)>>>(op->nx, op->ny, op->nz, op->w, op->shift,
                                                        xc, yc, w);
      break;
    case OPK_DIAG: {
      long want = (n + 255) / 256;
      long cap = (long)ctx->num_sms * 8 / w;
      if (cap < 4) cap = 4;
      if (want > cap) want = cap;
      dim3 grid((unsigned)want, w);
      if (f32)
        diag_kernel<float, float><<<grid, 256, 0, S(ctx)>>>(n, op->d32, xc, yc);
      else
        diag_kernel<double, double><<<grid, 256, 0, S(ctx)>>>(n, op->d, xc, yc);
      break;
    }
    default:
      return gb_fail(ctx, "unknown operator kind %d", op->kind);
  }
  gb_prof_end(ctx, &pr, bytes, flops);
  gb_count_launch(1);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "operator");
}

extern "C" void gpu_OperatorApply(void* op, void* X, void* Y)
{
  gpu_Operator* o = (gpu_Operator*)op;
  if (gb_operator_apply(o, (gpu_MultiVector*)X, (gpu_MultiVector*)Y)) {
    // the callback has no return value: the error stays in the context and
    // the solver checks it after the call
  }
}

// diagonal of the operator, on the host
__global__ void csr_diag_kernel(long n, const int* rowptr, const int* colidx, const double* vals,
                                double* out)
{
  long r = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (r >= n) return;
  double d = 0.0;
  for (int p = rowptr[r]; p < rowptr[r + 1]; p++)
    if (colidx[p] == r) d += vals[p];
  out[r] = d;
}

extern "C" int gpu_OperatorDiagonal(gpu_Operator* op, double* host_diag)
{
  gpu_Context* ctx = op->ctx;
  const long n = op->n;
  if (op->kind == OPK_DIAG) return gb_memcpy_d2h(ctx, host_diag, op->d, sizeof(double) * n);
  if (op->kind == OPK_CSR) {
    double* tmp = (double*)gb_device_alloc(ctx, sizeof(double) * n);
    if (!tmp) return -1;
    csr_diag_kernel<<<(unsigned)((n + 255) / 256), 256, 0, S(ctx)>>>(n, op->rowptr, op->colidx,
                                                                     op->vals, tmp);
    gb_count_launch(1);
    int rc = gb_cuda_check(ctx, (int)cudaGetLastError(), "csr_diag");
    if (!rc) rc = gb_memcpy_d2h(ctx, host_diag, tmp, sizeof(double) * n);
    gb_device_free(tmp);
    return rc;
  }
  // stencils: apply the operator to unit vectors is wasteful; sum on host
  if (op->kind == OPK_ST7 || op->kind == OPK_ST5) {
    int na = op->kind == OPK_ST7 ? 3 : 2;
    double* h[3] = {NULL, NULL, NULL};
    int rc = 0;
    for (int a = 0; a < na && !rc; a++) {
      h[a] = (double*)malloc(sizeof(double) * op->clen[a]);
      rc = gb_memcpy_d2h(ctx, h[a], op->c[a], sizeof(double) * op->clen[a]);
    }
    if (!rc) {
      const long nx = op->nx, ny = op->ny, nz = op->nz;
      for (long k = 0; k < nz; k++)
        for (long j = 0; j < ny; j++)
          for (long i = 0; i < nx; i++) {
            long c = i + nx * (j + ny * k);
            double s = op->shift + h[0][i + (nx + 1) * (j + ny * k)] +
                       h[0][i + 1 + (nx + 1) * (j + ny * k)] + h[1][i + nx * (j + (ny + 1) * k)] +
                       h[1][i + nx * (j + 1 + (ny + 1) * k)];
            if (na == 3) s += h[2][c] + h[2][c + nx * ny];
            host_diag[c] = s;
          }
    }
    for (int a = 0; a < na; a++) free(h[a]);
    return rc;
  }
  if (op->kind == OPK_ST27) {
    double* hw = (double*)malloc(sizeof(double) * n * 13);
    int rc = gb_memcpy_d2h(ctx, hw, op->w, sizeof(double) * n * 13);
    if (!rc) {
      const long nx = op->nx, ny = op->ny, nz = op->nz;
      for (long c = 0; c < n; c++) host_diag[c] = op->shift;
      for (long k = 0; k < nz; k++)
        for (long j = 0; j < ny; j++)
          for (long i = 0; i < nx; i++) {
            long c = i + nx * (j + ny * k);
            for (int e = 0; e < 13; e++) {
              long i2 = i + h_st27_off[e][0], j2 = j + h_st27_off[e][1], k2 = k + h_st27_off[e][2];
              if (i2 < 0 || i2 >= nx || j2 < 0 || j2 >= ny || k2 < 0 || k2 >= nz) continue;
              long d = i2 + nx * (j2 + ny * k2);
              host_diag[c] += hw[(size_t)e * n + c];
              host_diag[d] += hw[(size_t)e * n + c];
            }
          }
    }
    free(hw);
    return rc;
  }
  return gb_fail(ctx, "operator diagonal: unknown kind");
}

// ------------------------------------------------------------------------
// Parameter gradients of sum_i w_i' A x_i (the adjoint contraction of the
// eigenvalue / eigenvector derivatives): A is linear in its parameters, so
// d/dtheta = sum_i w_i' (dA/dtheta) x_i, evaluated per parameter.  W holds
// w_i = g_lambda_i x_i + mu_i (the output of gpu_EigenvectorAdjoint).
// No counterpart in the reference (it has no derivatives).
// ------------------------------------------------------------------------

// sum_i (w_i[p] - w_i[q]) (x_i[p] - x_i[q]): a coupling of weight c between p
// and q contributes c (e_p - e_q)(e_p - e_q)' to A; q < 0: c e_p e_p'
__device__ __forceinline__ double grad_pair(const blk_cols& X, const blk_cols& W, int k, long p,
                                            long q)
{
  double s = 0.0;
  for (int i = 0; i < k; i++) {
    const double* x = (const double*)X.col[i];
    const double* w = (const double*)W.col[i];
    if (q >= 0)
      s += (w[p] - w[q]) * (x[p] - x[q]);
    else
      s += w[p] * x[p];
  }
  return s;
}

__global__ void grad_csr_kernel(long n, const int* __restrict__ rowptr, const int* __restrict__ colidx,
                                blk_cols X, blk_cols W, int k, double* __restrict__ g)
{
  const long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (p >= n) return;
  for (int e = rowptr[p]; e < rowptr[p + 1]; e++) {
    const long q = colidx[e];
    double s = 0.0;
    for (int i = 0; i < k; i++) s += ((const double*)W.col[i])[p] * ((const double*)X.col[i])[q];
    g[e] = s;
  }
}

// faces of one direction of a grid stencil: face f = (a, b, c) with the face
// coordinate `a` along the direction in [0, na]; cells (a-1) and a
__global__ void grad_faces_kernel(int nx, int ny, int nz, int dir, blk_cols X, blk_cols W, int k,
                                  double* __restrict__ g)
{
  const int ex = nx + (dir == 0), ey = ny + (dir == 1), ez = nz + (dir == 2);
  const long nf = (long)ex * ey * ez;
  const long f = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int i = (int)(f % ex), j = (int)((f / ex) % ey), l = (int)(f / ((long)ex * ey));
  const int a = dir == 0 ? i : (dir == 1 ? j : l);
  const int na = dir == 0 ? nx : (dir == 1 ? ny : nz);
  const long stride = dir == 0 ? 1 : (dir == 1 ? (long)nx : (long)nx * ny);
  const long cell_hi = (long)(dir == 0 ? (i < nx ? i : nx - 1) : i) +
                       (long)nx * ((dir == 1 ? (j < ny ? j : ny - 1) : j) +
                                   (long)ny * (dir == 2 ? (l < nz ? l : nz - 1) : l));
  double s;
  if (a == 0)
    s = grad_pair(X, W, k, cell_hi, -1);
  else if (a == na)
    s = grad_pair(X, W, k, cell_hi, -1);  // cell_hi is the last cell here
  else
    s = grad_pair(X, W, k, cell_hi - stride, cell_hi);
  g[f] = s;
}

__global__ void grad_st27_kernel(int nx, int ny, int nz, blk_cols X, blk_cols W, int k,
                                 double* __restrict__ g)
{
  const long n = (long)nx * ny * nz;
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= n * 13) return;
  const long c = t / 13;
  const int e = (int)(t % 13);
  const int i = (int)(c % nx), j = (int)((c / nx) % ny), l = (int)(c / ((long)nx * ny));
  const int di = c_st27_off[e][0], dj = c_st27_off[e][1], dk = c_st27_off[e][2];
  const int i2 = i + di, j2 = j + dj, l2 = l + dk;
  double s = 0.0;
  if (i2 >= 0 && i2 < nx && j2 >= 0 && j2 < ny && l2 >= 0 && l2 < nz)
    s = grad_pair(X, W, k, c, c + di + (long)nx * (dj + (long)ny * dk));
  g[t] = s;  // cell-major, as the weights passed to gpu_Stencil27Create
}

__global__ void grad_diag_kernel(long n, blk_cols X, blk_cols W, int k, const double* lam,
                                 const double* xg, double* __restrict__ g)
{
  const long p = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (p >= n) return;
  double s = 0.0;
  for (int i = 0; i < k; i++) {
    const double x = ((const double*)X.col[i])[p], w = ((const double*)W.col[i])[p];
    s += lam ? -lam[i] * w * x - 0.5 * xg[i] * x * x : w * x;
  }
  g[p] = s;
}

static int grad_common(gpu_Operator* op, gpu_MultiVector* X, gpu_MultiVector* W, blk_cols* xc,
                       blk_cols* wc)
{
  gpu_Context* ctx = op->ctx;
  if (X->dtype != GPU_MV_FLOAT64 || W->dtype != GPU_MV_FLOAT64)
    return gb_fail(ctx, "operator gradient: FP64 blocks expected");
  if (X->size != op->n || W->size != op->n || X->num_active != W->num_active)
    return gb_fail(ctx, "operator gradient: block sizes do not match the operator");
  gb_mv_fill_cols(X, xc, 0);
  gb_mv_fill_cols(W, wc, 0);
  return 0;
}

extern "C" long gpu_OperatorParameterCount(gpu_Operator* op)
{
  switch (op->kind) {
    case OPK_CSR: return op->nnz;
    case OPK_ST7: return op->clen[0] + op->clen[1] + op->clen[2];
    case OPK_ST5: return op->clen[0] + op->clen[1];
    case OPK_ST27: return op->n * 13;
    case OPK_DIAG: return op->n;
  }
  return -1;
}

extern "C" int gpu_OperatorGradient(gpu_Operator* op, gpu_MultiVector* X, gpu_MultiVector* W,
                                    double* grad_host)
{
  gpu_Context* ctx = op->ctx;
  blk_cols xc, wc;
  if (grad_common(op, X, W, &xc, &wc)) return -1;
  const int k = X->num_active;
  const long np = gpu_OperatorParameterCount(op);
  double* g = (double*)gb_device_alloc(ctx, sizeof(double) * (size_t)(np > 0 ? np : 1));
  if (!g) return -1;
  const long n = op->n;
  int launches = 1;
  switch (op->kind) {
    case OPK_CSR:
      grad_csr_kernel<<<(unsigned)((n + 255) / 256), 256, 0, S(ctx)>>>(n, op->rowptr, op->colidx, xc,
                                                                        wc, k, g);
      break;
    case OPK_ST7:
    case OPK_ST5: {
      const int dirs = op->kind == OPK_ST7 ? 3 : 2;
      long off = 0;
      for (int d = 0; d < dirs; d++) {
        grad_faces_kernel<<<(unsigned)((op->clen[d] + 255) / 256), 256, 0, S(ctx)>>>(
            op->nx, op->ny, op->nz, d, xc, wc, k, g + off);
        off += op->clen[d];
      }
      launches = dirs;
      break;
    }
    case OPK_ST27:
      grad_st27_kernel<<<(unsigned)((n * 13 + 255) / 256), 256, 0, S(ctx)>>>(op->nx, op->ny, op->nz,
                                                                             xc, wc, k, g);
      break;
    case OPK_DIAG:
      grad_diag_kernel<<<(unsigned)((n + 255) / 256), 256, 0, S(ctx)>>>(n, xc, wc, k, NULL, NULL, g);
      break;
  }
  gb_count_launch(launches);
  int rc = gb_cuda_check(ctx, (int)cudaGetLastError(), "operator gradient");
  if (!rc) rc = gb_memcpy_d2h(ctx, grad_host, g, sizeof(double) * (size_t)np);
  gb_sync(ctx);
  gb_device_free(g);
  return rc;
}

extern "C" int gpu_MassGradient(gpu_Operator* B, gpu_MultiVector* X, gpu_MultiVector* W,
                                const double* lambda, const double* xg, double* grad_host)
{
  gpu_Context* ctx = B->ctx;
  if (B->kind != OPK_DIAG) return gb_fail(ctx, "mass gradient: B must be a diagonal operator");
  blk_cols xc, wc;
  if (grad_common(B, X, W, &xc, &wc)) return -1;
  const int k = X->num_active;
  const long n = B->n;
  double* g = (double*)gb_device_alloc(ctx, sizeof(double) * ((size_t)n + 2 * (size_t)k));
  if (!g) return -1;
  double* lam = g + n;
  double* xgd = lam + k;
  int rc = gb_memcpy_h2d(ctx, lam, lambda, sizeof(double) * k);
  if (!rc) {
    if (xg)
      rc = gb_memcpy_h2d(ctx, xgd, xg, sizeof(double) * k);
    else
      rc = cudaMemsetAsync(xgd, 0, sizeof(double) * k, S(ctx)) == cudaSuccess ? 0 : -1;
  }
  if (!rc) {
    grad_diag_kernel<<<(unsigned)((n + 255) / 256), 256, 0, S(ctx)>>>(n, xc, wc, k, lam, xgd, g);
    gb_count_launch(1);
    rc = gb_cuda_check(ctx, (int)cudaGetLastError(), "mass gradient");
  }
  if (!rc) rc = gb_memcpy_d2h(ctx, grad_host, g, sizeof(double) * (size_t)n);
  gb_sync(ctx);
  gb_device_free(g);
  return rc;
}

// ------------------------------------------------------------------------
// Inner conjugate-gradient preconditioner T ~ inv(A): Y = `iters` steps of
// (preconditioned) CG on A Y = X from Y = 0, every column an independent
// recurrence, all columns in lockstep (one block application of A per
// step).  The preconditioner of HYPRE's LOBPCG driver with -pcgitr
// (blopex_hypre/krylov/HYPRE_lobpcg.c:317-320, precondUsageMode): a fixed
// number of CG steps, so T is only approximately linear, which LOBPCG
// tolerates.  Works in the dtype of the blocks (FP32 in the FP32 phase).
// ------------------------------------------------------------------------
template <typename T>
__global__ void pcg_cols_kernel(long n, int mode, blk_cols A, blk_cols B, blk_cols C, blk_cols D,
                                const double* __restrict__ a)
{
  // mode 0: C_i = a_i A_i (first step: Y = alpha P), D_i -= a_i B_i
  // mode 1: C_i += a_i A_i,  D_i -= a_i B_i
  // mode 2: C_i = A_i + a_i C_i  (P = Z + beta P)
  const int i = blockIdx.y;
  const T ai = (T)a[i];
  const T* x = (const T*)A.col[i];
  const T* y = (const T*)B.col[i];
  T* c = (T*)C.col[i];
  T* d = (T*)D.col[i];
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    if (mode == 2) {
      c[r] = x[r] + ai * c[r];
    } else {
      c[r] = (mode == 0 ? T(0) : c[r]) + ai * x[r];
      d[r] -= ai * y[r];
    }
  }
}

__global__ void pcg_ratio_kernel(int k, const double* num, const double* den, double* out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) out[i] = (den[i] != 0.0 && num[i] != 0.0) ? num[i] / den[i] : 0.0;
}

// FP32 blocks with 16-byte aligned columns and a diagonal (Jacobi) or no
// inner preconditioner M: the column updates of a CG step fused with the
// inner product that follows them, float4 access, and z = M r recomputed
// where it is read instead of stored (M is one column, L2-resident).  Per
// step 13 block passes instead of 17.  Inner products as gb_dot_cols' FP32
// path (exact products, compensated FP32 sums flushed to FP64).
//   init: r = x ; p = M x ; partial x' M x
//   step: y = alpha p (first) or y += alpha p ; r -= alpha q ; partial r' M r
//   dir:  p = M r + beta p
template <bool HAVE_M>
static __device__ __forceinline__ float4 pcg32_m(const float4* m, long v, float4 r)
{
  if (!HAVE_M) return r;
  const float4 d = m[v];
  return make_float4(d.x * r.x, d.y * r.y, d.z * r.z, d.w * r.w);
}

template <bool HAVE_M>
__global__ void __launch_bounds__(256) pcg32_init_kernel(long n, blk_cols X, const float* __restrict__ m,
                                                         blk_cols R, blk_cols P,
                                                         double* __restrict__ partial)
{
  const float* x = (const float*)X.col[blockIdx.y];
  float* r = (float*)R.col[blockIdx.y];
  float* p = (float*)P.col[blockIdx.y];
  const long n4 = n >> 2, stride = (long)gridDim.x * blockDim.x;
  double acc = 0.0;
  float s = 0.f, c = 0.f;
  int cnt = 0;
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < n4; v += stride) {
    const float4 xv = ((const float4*)x)[v];
    const float4 z = pcg32_m<HAVE_M>((const float4*)m, v, xv);
    ((float4*)r)[v] = xv;
    ((float4*)p)[v] = z;
    acc_prod32x4(s, c, xv, z);
    if (++cnt == 16) {
      acc += (double)s + (double)c;
      s = c = 0.f;
      cnt = 0;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x < (n & 3)) {
    const long e = 4 * n4 + threadIdx.x;
    const float z = HAVE_M ? m[e] * x[e] : x[e];
    r[e] = x[e];
    p[e] = z;
    acc_prod32(s, c, x[e], z);
  }
  acc += (double)s + (double)c;
  const double t = block_sum256(acc);
  if (threadIdx.x == 0) partial[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = t;
}

template <bool HAVE_M, bool FIRST>
__global__ void __launch_bounds__(256) pcg32_step_kernel(long n, blk_cols P, blk_cols Q, blk_cols Y,
                                                         blk_cols R, const float* __restrict__ m,
                                                         const double* __restrict__ alpha,
                                                         double* __restrict__ partial)
{
  const int j = blockIdx.y;
  const float a = (float)alpha[j];
  const float* p = (const float*)P.col[j];
  const float* q = (const float*)Q.col[j];
  float* y = (float*)Y.col[j];
  float* r = (float*)R.col[j];
  const long n4 = n >> 2, stride = (long)gridDim.x * blockDim.x;
  double acc = 0.0;
  float s = 0.f, c = 0.f;
  int cnt = 0;
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < n4; v += stride) {
    const float4 pv = ((const float4*)p)[v], qv = ((const float4*)q)[v];
    float4 rv = ((float4*)r)[v];
    float4 yv;
    if (FIRST) {
      yv = make_float4(a * pv.x, a * pv.y, a * pv.z, a * pv.w);
    } else {
      yv = ((float4*)y)[v];
      yv = make_float4(fmaf(a, pv.x, yv.x), fmaf(a, pv.y, yv.y), fmaf(a, pv.z, yv.z), fmaf(a, pv.w, yv.w));
    }
    rv = make_float4(fmaf(-a, qv.x, rv.x), fmaf(-a, qv.y, rv.y), fmaf(-a, qv.z, rv.z), fmaf(-a, qv.w, rv.w));
    ((float4*)y)[v] = yv;
    ((float4*)r)[v] = rv;
    if (partial) {
      acc_prod32x4(s, c, rv, pcg32_m<HAVE_M>((const float4*)m, v, rv));
      if (++cnt == 16) {
        acc += (double)s + (double)c;
        s = c = 0.f;
        cnt = 0;
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x < (n & 3)) {
    const long e = 4 * n4 + threadIdx.x;
    y[e] = FIRST ? a * p[e] : fmaf(a, p[e], y[e]);
    const float re = fmaf(-a, q[e], r[e]);
    r[e] = re;
    if (partial) acc_prod32(s, c, re, HAVE_M ? m[e] * re : re);
  }
  if (!partial) return;  // uniform over the grid
  acc += (double)s + (double)c;
  const double t = block_sum256(acc);
  if (threadIdx.x == 0) partial[(size_t)j * gridDim.x + blockIdx.x] = t;
}

template <bool HAVE_M>
__global__ void __launch_bounds__(256) pcg32_dir_kernel(long n, blk_cols R, const float* __restrict__ m,
                                                        blk_cols P, const double* __restrict__ beta)
{
  const int j = blockIdx.y;
  const float b = (float)beta[j];
  const float* r = (const float*)R.col[j];
  float* p = (float*)P.col[j];
  const long n4 = n >> 2, stride = (long)gridDim.x * blockDim.x;
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < n4; v += stride) {
    const float4 z = pcg32_m<HAVE_M>((const float4*)m, v, ((const float4*)r)[v]);
    float4 pv = ((float4*)p)[v];
    pv = make_float4(fmaf(b, pv.x, z.x), fmaf(b, pv.y, z.y), fmaf(b, pv.z, z.z), fmaf(b, pv.w, z.w));
    ((float4*)p)[v] = pv;
  }
  if (blockIdx.x == 0 && threadIdx.x < (n & 3)) {
    const long e = 4 * n4 + threadIdx.x;
    p[e] = fmaf(b, p[e], HAVE_M ? m[e] * r[e] : r[e]);
  }
}

extern "C" gpu_Operator* gpu_PCGPreconditionerCreate(gpu_Context* ctx, gpu_Operator* A,
                                                     gpu_Operator* M, int iterations)
{
  if (!A || iterations < 1 || (M && M->n != A->n)) {
    gb_fail(ctx, "PCG preconditioner: bad arguments");
    return NULL;
  }
  gpu_Operator* op = op_new(ctx, OPK_PCG, A->n);
  op->inner = A;
  op->prec = M;
  op->iters = iterations;
  op->coef = (double*)gb_device_alloc(ctx, sizeof(double) * 4 * BLK_MAXCOLS);
  if (!op->coef) {
    gpu_OperatorDestroy(op);
    return NULL;
  }
  return op;
}

// the FP32 inner CG of pcg_apply on the fused kernels above (M diagonal or
// absent, aligned columns); the same recurrences and coefficients
static int pcg32_fused(gpu_Operator* op, gpu_MultiVector* X, const blk_cols* cx, const blk_cols* cy,
                       const blk_cols* cr, const blk_cols* cp, const blk_cols* cq, int w, dim3 grid,
                       const int* idx)
{
  gpu_Context* ctx = op->ctx;
  const long n = op->n;
  const float* m = op->prec ? op->prec->d32 : NULL;
  double *rho = op->coef, *rho2 = rho + BLK_MAXCOLS, *pq = rho2 + BLK_MAXCOLS, *al = pq + BLK_MAXCOLS;
  const double blk = 4.0 * (double)n * w, mb = m ? 4.0 * (double)n : 0.0;
  gpu_MultiVector* p = op->work[2];
  gpu_MultiVector* q = op->work[3];
  gb_prof_rec pr;
  // r = x ; p = M x ; rho = x' M x
  double* partial = (double*)gb_workspace(ctx, sizeof(double) * (size_t)grid.x * w);
  if (!partial) return -1;
  gb_prof_begin(ctx, &pr, GB_K_BLAS1);
  if (m)
    pcg32_init_kernel<true><<<grid, 256, 0, S(ctx)>>>(n, *cx, m, *cr, *cp, partial);
  else
    pcg32_init_kernel<false><<<grid, 256, 0, S(ctx)>>>(n, *cx, m, *cr, *cp, partial);
  gb_prof_end(ctx, &pr, 3.0 * blk + mb, 2.0 * n * w);
  gb_count_launch(1);
  if (gb_dot_reduce(ctx, partial, (int)grid.x, w, rho, idx)) return -1;
  (void)X;
  for (int it = 0; it < op->iters; it++) {
    // q = A p with p' q folded into the operator's kernel where it can be
    const int fused = gb_operator_apply_dot(op->inner, p, q, pq);
    if (fused < 0) return -1;
    if (fused == 1 && (gb_operator_apply(op->inner, p, q) ||
                       gb_dot_cols(ctx, GPU_MV_FLOAT32, n, cp, cq, w, pq, idx)))
      return -1;
    pcg_ratio_kernel<<<1, BLK_MAXCOLS, 0, S(ctx)>>>(w, rho, pq, al);
    gb_count_launch(1);
    const bool last = it + 1 == op->iters;
    partial = last ? NULL : (double*)gb_workspace(ctx, sizeof(double) * (size_t)grid.x * w);
    if (!last && !partial) return -1;
    gb_prof_begin(ctx, &pr, GB_K_BLAS1);
    if (it == 0) {
      if (m)
        pcg32_step_kernel<true, true><<<grid, 256, 0, S(ctx)>>>(n, *cp, *cq, *cy, *cr, m, al, partial);
      else
        pcg32_step_kernel<false, true><<<grid, 256, 0, S(ctx)>>>(n, *cp, *cq, *cy, *cr, m, al, partial);
    } else {
      if (m)
        pcg32_step_kernel<true, false><<<grid, 256, 0, S(ctx)>>>(n, *cp, *cq, *cy, *cr, m, al, partial);
      else
        pcg32_step_kernel<false, false><<<grid, 256, 0, S(ctx)>>>(n, *cp, *cq, *cy, *cr, m, al, partial);
    }
    gb_prof_end(ctx, &pr, (it == 0 ? 5.0 : 6.0) * blk + (last ? 0.0 : mb), 4.0 * n * w);
    gb_count_launch(1);
    if (last) break;
    if (gb_dot_reduce(ctx, partial, (int)grid.x, w, rho2, idx)) return -1;
    pcg_ratio_kernel<<<1, BLK_MAXCOLS, 0, S(ctx)>>>(w, rho2, rho, al);  // beta
    gb_count_launch(1);
    gb_prof_begin(ctx, &pr, GB_K_BLAS1);
    if (m)
      pcg32_dir_kernel<true><<<grid, 256, 0, S(ctx)>>>(n, *cr, m, *cp, al);
    else
      pcg32_dir_kernel<false><<<grid, 256, 0, S(ctx)>>>(n, *cr, m, *cp, al);
    gb_prof_end(ctx, &pr, 3.0 * blk + mb, 2.0 * n * w);
    gb_count_launch(1);
    double* t = rho;
    rho = rho2;
    rho2 = t;
  }
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "pcg preconditioner");
}

static int pcg_apply(gpu_Operator* op, gpu_MultiVector* X, gpu_MultiVector* Y)
{
  gpu_Context* ctx = op->ctx;
  const int w = X->num_active;
  if (X->size != op->n || Y->size != op->n || Y->num_active != w || X->dtype != Y->dtype)
    return gb_fail(ctx, "PCG preconditioner: block shapes");
  if (w == 0) return 0;
  if (X->dtype == GPU_MV_FLOAT64 && ctx->opt.precision == LOBPCG_GPU_MIXED &&
      ctx->opt.fp32_precond) {
    // mixed mode, FP64 block: the inner iteration on FP32 copies.  The
    // preconditioner only shapes the search direction T r (the solver's
    // residuals and Ritz pairs stay FP64), and on this GPU an FP64 operator
    // application is FP64-pipe bound where the FP32 one is HBM bound.
    gpu_MultiVector** io = op->io32;
    if (!io[0] || io[0]->num_vectors < w) {
      for (int b = 0; b < 2; b++) {
        gpu_MultiVectorDestroy(io[b]);
        io[b] = gpu_MultiVectorCreate(ctx, op->n, w, GPU_MV_FLOAT32);
        if (!io[b]) return -1;
      }
    }
    int mask[BLK_MAXCOLS];
    for (int c = 0; c < io[0]->num_vectors; c++) mask[c] = c < w;
    gb_mv_set_mask_host(io[0], mask);
    gb_mv_set_mask_host(io[1], mask);
    blk_cols cx, cy, c0, c1;
    gb_mv_fill_cols(X, &cx, 0);
    gb_mv_fill_cols(Y, &cy, 0);
    gb_mv_fill_cols(io[0], &c0, 0);
    gb_mv_fill_cols(io[1], &c1, 0);
    if (gb_convert(ctx, op->n, GPU_MV_FLOAT64, &cx, GPU_MV_FLOAT32, &c0, w)) return -1;
    if (pcg_apply(op, io[0], io[1])) return -1;
    return gb_convert(ctx, op->n, GPU_MV_FLOAT32, &c1, GPU_MV_FLOAT64, &cy, w);
  }
  // work blocks of (at least) this width and dtype
  gpu_MultiVector** wk = op->work;
  if (!wk[0] || wk[0]->dtype != X->dtype || wk[0]->num_vectors < w) {
    for (int b = 0; b < 4; b++) {
      gpu_MultiVectorDestroy(wk[b]);
      wk[b] = gpu_MultiVectorCreate(ctx, op->n, w, X->dtype);
      if (!wk[b]) return -1;
    }
  }
  int mask[BLK_MAXCOLS];
  const int nv = wk[0]->num_vectors;
  for (int c = 0; c < nv; c++) mask[c] = c < w;
  for (int b = 0; b < 4; b++) gb_mv_set_mask_host(wk[b], mask);
  gpu_MultiVector *r = wk[0], *z = wk[1], *p = wk[2], *q = wk[3];
  blk_cols cx, cy, cr, cz, cp, cq;
  gb_mv_fill_cols(X, &cx, 0);
  gb_mv_fill_cols(Y, &cy, 0);
  gb_mv_fill_cols(r, &cr, 0);
  gb_mv_fill_cols(z, &cz, 0);
  gb_mv_fill_cols(p, &cp, 0);
  gb_mv_fill_cols(q, &cq, 0);
  double *rho = op->coef, *rho2 = rho + BLK_MAXCOLS, *pq = rho2 + BLK_MAXCOLS,
         *al = pq + BLK_MAXCOLS;
  int idx[BLK_MAXCOLS];
  for (int c = 0; c < w; c++) idx[c] = c;
  const int dt = X->dtype;
  const int f32 = dt == GPU_MV_FLOAT32;
  long want = (op->n + 255) / 256, cap = (long)ctx->num_sms * 8 / w;
  if (cap < 4) cap = 4;
  if (want > cap) want = cap;
  const dim3 grid((unsigned)want, w);
  const bool mdiag = !op->prec || op->prec->kind == OPK_DIAG;
  if (f32 && mdiag && cols_aligned16(cx.col, w) && cols_aligned16(cy.col, w) &&
      cols_aligned16(cr.col, w) && cols_aligned16(cp.col, w) && cols_aligned16(cq.col, w) &&
      (!op->prec || ensure_f32(op->prec) == 0)) {
    // the inner products A p with FP64 coefficients and arithmetic when the
    // context asks for accurate FP32 operators
    const int acc_saved = ctx->op_accurate;
    if (ctx->opt.fp32_accurate_op) ctx->op_accurate = 1;
    const int rc = pcg32_fused(op, X, &cx, &cy, &cr, &cp, &cq, w, grid, idx);
    ctx->op_accurate = acc_saved;
    return rc;
  }
#define PCG_COLS(mode, a, b, c, d, coef)                                                    \
  do {                                                                                    \
    if (f32)                                                                              \
      pcg_cols_kernel<float><<<grid, 256, 0, S(ctx)>>>(op->n, mode, a, b, c, d, coef);    \
    else                                                                                  \
      pcg_cols_kernel<double><<<grid, 256, 0, S(ctx)>>>(op->n, mode, a, b, c, d, coef);   \
    gb_count_launch(1);                                                                   \
  } while (0)
  // r = x ; z = M r ; p = z ; rho = r'z
  if (gb_axpby(ctx, dt, op->n, 1.0, &cx, 0.0, &cr, w)) return -1;
  if (op->prec) {
    if (gb_operator_apply(op->prec, r, z)) return -1;
  } else if (gb_axpby(ctx, dt, op->n, 1.0, &cr, 0.0, &cz, w)) {
    return -1;
  }
  if (gb_axpby(ctx, dt, op->n, 1.0, &cz, 0.0, &cp, w)) return -1;
  if (gb_dot_cols(ctx, dt, op->n, &cr, &cz, w, rho, idx)) return -1;
  // FP32 blocks: the inner products A p with FP64 coefficients and
  // arithmetic when the context asks for accurate FP32 operators
  const int acc_saved = ctx->op_accurate;
  if (f32 && ctx->opt.fp32_accurate_op) ctx->op_accurate = 1;
  for (int it = 0; it < op->iters; it++) {
    const int rca = gb_operator_apply(op->inner, p, q);
    if (rca) {
      ctx->op_accurate = acc_saved;
      { ctx->op_accurate = acc_saved; return -1; }
    }
    if (gb_dot_cols(ctx, dt, op->n, &cp, &cq, w, pq, idx)) { ctx->op_accurate = acc_saved; return -1; }
    pcg_ratio_kernel<<<1, BLK_MAXCOLS, 0, S(ctx)>>>(w, rho, pq, al);
    gb_count_launch(1);
    PCG_COLS(it == 0 ? 0 : 1, cp, cq, cy, cr, al);  // y += alpha p ; r -= alpha q
    if (it + 1 == op->iters) break;
    if (op->prec) {
      if (gb_operator_apply(op->prec, r, z)) { ctx->op_accurate = acc_saved; return -1; }
    } else if (gb_axpby(ctx, dt, op->n, 1.0, &cr, 0.0, &cz, w)) {
      { ctx->op_accurate = acc_saved; return -1; }
    }
    if (gb_dot_cols(ctx, dt, op->n, &cr, &cz, w, rho2, idx)) { ctx->op_accurate = acc_saved; return -1; }
    pcg_ratio_kernel<<<1, BLK_MAXCOLS, 0, S(ctx)>>>(w, rho2, rho, al);  // beta
    gb_count_launch(1);
    PCG_COLS(2, cz, cz, cp, cp, al);  // p = z + beta p
    double* t = rho;
    rho = rho2;
    rho2 = t;
  }
#undef PCG_COLS
  ctx->op_accurate = acc_saved;
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "pcg preconditioner");
}
