// tiles.cu -- tile work items of one instance, 16-bit halo slots of every bond, FP32
// position records and the sliced operator (32 rows per slice, column-major, each bond
// column 32 FP32 weights + 32 16-bit codes) that the FP32 kernels stream.
//
// A tile is T consecutive bins along x (bins of side >= the horizon radius, x-fastest
// order, so the tile's own nodes and each of its 3x3 halo rows are contiguous node
// ranges).  A kernel stages a tile's halo into shared memory and reaches a neighbour through
// its slot: the neighbour's position in the concatenation of the halo rows.
#include <algorithm>
#include <cstring>
#include <vector>

#include "engine.cuh"

namespace nnpp {

namespace {

struct Grid3 {
  int nb[3];
  int T;
};

// halo rows r = (dy+1) + 3 (dz+1) of tile (tx, by, bz): node ranges [hb, hb+hl)
__host__ __device__ inline void tile_rows(const int* bin_start, Grid3 g, int tx, int by, int bz,
                                          int* hb, int* hl) {
  const int lo = max(tx * g.T - 1, 0);
  const int hi = min(tx * g.T + g.T, g.nb[0] - 1);
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy) {
      const int r = (dy + 1) + 3 * (dz + 1);
      const int yy = by + dy, zz = bz + dz;
      if (yy < 0 || yy >= g.nb[1] || zz < 0 || zz >= g.nb[2]) {
        hb[r] = 0;
        hl[r] = 0;
        continue;
      }
      const int b0 = lo + g.nb[0] * (yy + g.nb[1] * zz);
      const int b1 = hi + g.nb[0] * (yy + g.nb[1] * zz);
      hb[r] = bin_start[b0];
      hl[r] = bin_start[b1 + 1] - bin_start[b0];
    }
}

__global__ void k_posrec(int n, const double* pos, double ox, double oy, double oz, double hb,
                         int nbx, int nby, int nbz, float4* rec) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
    const double x = pos[a], y = pos[n + a], z = pos[2 * n + a];
    int bx = (int)((x - ox) / hb), by = (int)((y - oy) / hb), bz = (int)((z - oz) / hb);
    bx = min(max(bx, 0), nbx - 1);
    by = min(max(by, 0), nby - 1);
    bz = min(max(bz, 0), nbz - 1);
    float4 r;
    r.x = (float)(x - (ox + (double)bx * hb));
    r.y = (float)(y - (oy + (double)by * hb));
    r.z = (float)(z - (oz + (double)bz * hb));
    r.w = __int_as_float(bx | (by << 10) | (bz << 20));
    rec[a] = r;
  }
}

// warp per node: slot of every neighbour within the halo of the node's tile
__global__ void k_slots(int n, const int* row, const int* col, const float4* posrec,
                        const int* bin_start, Grid3 g, unsigned short* slot, int* err) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; a < n; a += warps) {
    const int pb = __float_as_int(posrec[a].w);
    const int bx = pb & 1023, by = (pb >> 10) & 1023, bz = (pb >> 20) & 1023;
    int hb[9], hl[9], off[9];
    tile_rows(bin_start, g, bx / g.T, by, bz, hb, hl);
    int acc = 0;
    for (int r = 0; r < 9; ++r) {
      off[r] = acc;
      acc += hl[r];
    }
    for (int j = row[a] + lane; j < row[a + 1]; j += 32) {
      const int nn = col[j];
      const int q = __float_as_int(posrec[nn].w);
      const int dy = ((q >> 10) & 1023) - by, dz = ((q >> 20) & 1023) - bz;
      int s = -1;
      if (dy >= -1 && dy <= 1 && dz >= -1 && dz <= 1) {
        const int r = (dy + 1) + 3 * (dz + 1);
        if (nn >= hb[r] && nn < hb[r] + hl[r]) s = off[r] + (nn - hb[r]);
      }
      if (s < 0 || s > 65535) {
        atomicExch(err, 1);
        s = 0;
      }
      slot[j] = (unsigned short)s;
    }
  }
}

// node of a tile-halo slot: pre = starts of the tile's 9 halo rows in its halo, hb = their
// first nodes
__device__ __forceinline__ void slot_node(int sv, const int* pre, const int* hb, int* r, int* node) {
  int q = 0;
  while (q < 8 && sv >= pre[q + 1]) ++q;
  *r = q;
  *node = hb[q] + (sv - pre[q]);
}

// warp per slice: the node range [lo, hi) each of the 9 halo rows contributes to the slice
__global__ void k_slice_windows(int nslices, const SliceDesc* sl, const int* pre_hb, const int* row,
                                const unsigned short* slot, int* lohi) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += warps) {
    const SliceDesc d = sl[s];
    const int* pre = pre_hb + 18 * s;
    const int* hb = pre + 9;
    int lo[9], hi[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      lo[q] = 0x7fffffff;
      hi[q] = -1;
    }
    if (lane < d.nrows) {
      const int j1 = row[d.row0 + lane + 1];
      for (int j = row[d.row0 + lane]; j < j1; ++j) {
        int r, node;
        slot_node(slot[j], pre, hb, &r, &node);
#pragma unroll
        for (int q = 0; q < 9; ++q)
          if (q == r) {
            lo[q] = min(lo[q], node);
            hi[q] = max(hi[q], node + 1);
          }
      }
    }
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      lo[q] = __reduce_min_sync(0xffffffffu, lo[q]);
      hi[q] = __reduce_max_sync(0xffffffffu, hi[q]);
    }
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        lohi[18 * s + q] = lo[q];
        lohi[18 * s + 9 + q] = hi[q];
      }
  }
}

// warp per slice: bond c of lane l (row row0 + l): its FP32 weight at float 48 (off/32 + c)
// + l of the interleaved array, its code (window row << 12 | node - gbase[row]) at 16-bit
// element 96 (off/32 + c) + 64 + l; padding: code 0, weight 0
__global__ void k_sell_fill(int nslices, const SliceDesc* sl, const int* pre_hb, const int* row,
                            const unsigned short* slot, const float* w32, const float* wlo32, float* sell,
                            float* sell_lo) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += warps) {
    const SliceDesc& d = sl[s];
    const int* pre = pre_hb + 18 * s;
    const int* hb = pre + 9;
    const bool live = lane < d.nrows;
    const int j0 = live ? row[d.row0 + lane] : 0;
    const int len = live ? row[d.row0 + lane + 1] - j0 : 0;
    for (int c = 0; c < d.width; ++c) {
      float* col = sell + ((size_t)(d.off >> 5) + c) * 48;
      unsigned short code = 0;
      float w = 0.0f, wl = 0.0f;
      if (c < len) {
        int r, node;
        slot_node(slot[j0 + c], pre, hb, &r, &node);
        code = (unsigned short)((r << 12) | (node - d.gbase[r]));
        w = w32[j0 + c];
        wl = wlo32[j0 + c];
      }
      col[lane] = w;
      reinterpret_cast<unsigned short*>(col + 32)[lane] = code;
      sell_lo[((size_t)(d.off >> 5) + c) * 32 + lane] = wl;
    }
  }
}

// warp per CG slice: the node range [lo, hi) of its rows' neighbours without a potential
// Dirichlet value in each of the 9 window rows (the bin rows by + dy, bz + dz, dy, dz in
// -1..1, row (dy + 1) + 3 (dz + 1))
__global__ void k_cg_windows(int nslices, const SliceDesc* sl, const int* cg_rows, const int* row,
                             const int* col, const unsigned char* dirmask, const int* xrow, int* lohi) {
  constexpr unsigned char kPhiDir = 1u << S;
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += warps) {
    const SliceDesc& d = sl[s];
    const int by = d.tile & 0xffff, bz = d.tile >> 16;
    int lo[9], hi[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      lo[q] = 0x7fffffff;
      hi[q] = -1;
    }
    const int a = lane < d.nrows ? cg_rows[d.row0 + lane] : -1;
    if (a >= 0)
      for (int j = row[a]; j < row[a + 1]; ++j) {
        const int m = col[j];
        if (dirmask[m] & kPhiDir) continue;
        const int xr = xrow[m];
        const int r = ((xr & 0xffff) - by + 1) + 3 * ((xr >> 16) - bz + 1);
#pragma unroll
        for (int q = 0; q < 9; ++q)
          if (q == r) {
            lo[q] = min(lo[q], m);
            hi[q] = max(hi[q], m + 1);
          }
      }
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      lo[q] = __reduce_min_sync(0xffffffffu, lo[q]);
      hi[q] = __reduce_max_sync(0xffffffffu, hi[q]);
    }
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        lohi[18 * s + q] = lo[q];
        lohi[18 * s + 9 + q] = hi[q];
      }
  }
}

// per node: -1 for a node with a Dirichlet value of the potential, else its number of
// neighbours without one (the row length of the halo-staged CG operator)
__global__ void k_omega_degree(int n, const int* row, const int* col, const unsigned char* dirmask,
                               int* deg) {
  constexpr unsigned char kPhiDir = 1u << S;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
    if (dirmask[a] & kPhiDir) {
      deg[a] = -1;
      continue;
    }
    int d = 0;
    for (int j = row[a]; j < row[a + 1]; ++j) d += (dirmask[col[j]] & kPhiDir) ? 0 : 1;
    deg[a] = d;
  }
}

// thread per (quad, row): the row's codes in CSR order (ascending halo slot), then the
// tile's padding slot up to the quad's pass count
__global__ void k_fill_hcode(int nquads, const HQuad* quads, const int* row, const int* col,
                             const unsigned short* slot16, const unsigned char* dirmask,
                             unsigned short* code) {
  constexpr unsigned char kPhiDir = 1u << S;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < 4 * nquads; idx += gridDim.x * blockDim.x) {
    const HQuad q = quads[idx >> 2];
    const int g = idx & 3;
    const int a = q.rows[g];
    const int base = q.coff_abs + 8 * g;
    const int total = 8 * q.npass;
    int m = 0;
    if (a >= 0)
      for (int j = row[a]; j < row[a + 1] && m < total; ++j)
        if (!(dirmask[col[j]] & kPhiDir)) {
          code[base + 32 * (m >> 3) + (m & 7)] = slot16[j];
          ++m;
        }
    for (; m < total; ++m) code[base + 32 * (m >> 3) + (m & 7)] = (unsigned short)q.padcode;
  }
}

}  // namespace

nnpp_status build_tiles(Handle& h, int T, std::vector<TileDesc>& tiles, std::vector<SliceDesc>& gslices,
                        int inst, int* halo_max, int* bond_max, bool* windows_fit) {
  const Layout& L = h.lay;
  const int N = h.N;
  if (L.nb[0] > 1024 || L.nb[1] > 1024 || L.nb[2] > 1024)
    return set_error(NNPP_ERR_UNSUPPORTED, "tiles: more than 1024 bins per axis");
  Grid3 g;
  g.nb[0] = L.nb[0];
  g.nb[1] = L.nb[1];
  g.nb[2] = L.nb[2];
  g.T = T;
  const double hb = (double)h.h32;
  // slots are staged per tile with 16-byte loads from a multiple of 8: pad the array
  if (!h.posrec.alloc(N) || !h.slot16.alloc((size_t)L.nnz + 16))
    return set_error(NNPP_ERR_NOMEM, "tile arrays");
  NNPP_CUDA(cudaMemsetAsync(h.slot16.get(), 0, sizeof(unsigned short) * ((size_t)L.nnz + 16), h.st));
  const int blocks = std::max(1, std::min((N + 255) / 256, 152 * 16));
  k_posrec<<<blocks, 256, 0, h.st>>>(N, L.pos.get(), h.ref.bbox[0], h.ref.bbox[2], h.ref.bbox[4], hb,
                                     g.nb[0], g.nb[1], g.nb[2], h.posrec.get());
  DBuf<int> err;
  if (!err.alloc(1)) return set_error(NNPP_ERR_NOMEM, "tile flag");
  NNPP_CUDA(cudaMemsetAsync(err.get(), 0, sizeof(int), h.st));
  const int wblocks = std::max(1, std::min((int)(((long long)N * 32 + 255) / 256), 152 * 64));
  k_slots<<<wblocks, 256, 0, h.st>>>(N, L.row.get(), L.col.get(), h.posrec.get(), L.bin_start.get(), g,
                                     h.slot16.get(), err.get());
  NNPP_CUDA(cudaGetLastError());
  std::vector<int> bs(L.nbins + 1), rows(N + 1);
  int herr = 0;
  NNPP_CUDA(cudaMemcpyAsync(bs.data(), L.bin_start.get(), sizeof(int) * (L.nbins + 1), cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaMemcpyAsync(rows.data(), L.row.get(), sizeof(int) * (N + 1), cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaMemcpyAsync(&herr, err.get(), sizeof(int), cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  if (herr) return set_error(NNPP_ERR_INVALID, "tiles: a neighbour outside its tile's halo");
  const int ntx = (g.nb[0] + T - 1) / T;
  int hm = 0, bm = 0;
  std::vector<SliceDesc> slices;  // this instance's, offsets local to its sliced arrays
  std::vector<int> pre;            // per slice: starts of the 9 halo rows in the halo, then
                                   // their first nodes (18 ints)
  long long soff = 0;
  for (int bz = 0; bz < g.nb[2]; ++bz)
    for (int by = 0; by < g.nb[1]; ++by)
      for (int tx = 0; tx < ntx; ++tx) {
        const int bx0 = tx * T, bx1 = std::min(tx * T + T, g.nb[0]) - 1;
        const int o0 = bs[bx0 + g.nb[0] * (by + g.nb[1] * bz)];
        const int o1 = bs[bx1 + g.nb[0] * (by + g.nb[1] * bz) + 1];
        if (o1 <= o0) continue;
        TileDesc t;
        t.inst = inst;
        t.own_begin = o0;
        t.own_end = o1;
        tile_rows(bs.data(), g, tx, by, bz, t.hb, t.hl);
        int tot = 0;
        for (int r = 0; r < 9; ++r) tot += t.hl[r];
        if (tot > 65536) return set_error(NNPP_ERR_UNSUPPORTED, "tiles: halo larger than 65536 nodes");
        t.halo = tot;
        t.slice0 = (int)(gslices.size() + slices.size());
        t.pad[0] = t.pad[1] = 0;
        for (int r = 0; r < 9; ++r)
          if (t.hl[r] > 4096) return set_error(NNPP_ERR_UNSUPPORTED, "tiles: halo row longer than 4096 nodes");
        for (int r0 = o0; r0 < o1; r0 += 32) {
          SliceDesc d;
          d.inst = inst;
          d.tile = (int)tiles.size();
          d.row0 = r0;
          d.nrows = std::min(32, o1 - r0);
          d.off = (int)soff;
          d.width = 0;
          d.wtotal = d.pad = 0;
          for (int q = 0; q < 4; ++q) d.pad2[q] = 0;
          for (int r = 0; r < 9; ++r) d.lo[r] = d.woff[r] = d.wlen[r] = d.gbase[r] = 0;
          for (int l = 0; l < d.nrows; ++l) d.width = std::max(d.width, rows[r0 + l + 1] - rows[r0 + l]);
          slices.push_back(d);
          int acc = 0;
          for (int r = 0; r < 9; ++r) {
            pre.push_back(acc);
            acc += t.hl[r];
          }
          for (int r = 0; r < 9; ++r) pre.push_back(t.hb[r]);
          soff += 32LL * d.width;
          if (soff > 0x7fffffffLL) return set_error(NNPP_ERR_UNSUPPORTED, "sliced operator above 2^31 entries");
        }
        t.bond0 = rows[o0] & ~7;
        t.bond1 = rows[o1];
        hm = std::max(hm, tot);
        bm = std::max(bm, t.bond1 - t.bond0);
        tiles.push_back(t);
      }
  // sliced copy of the slot codes and FP32 weights for the CG operator and the transport
  const size_t ns = slices.size();
  if (!h.sell.alloc((size_t)(soff / 32) * 48 + 48) || !h.sell_lo.alloc((size_t)(soff / 32) * 32 + 32))
    return set_error(NNPP_ERR_NOMEM, "sliced operator");
  DBuf<SliceDesc> dsl;
  DBuf<int> dpre, dlohi;
  bool fit = true;
  if (ns && (!dsl.alloc(ns) || !dpre.alloc(18 * ns) || !dlohi.alloc(18 * ns)))
    return set_error(NNPP_ERR_NOMEM, "sliced operator");
  if (ns) {
    NNPP_CUDA(cudaMemcpyAsync(dsl.get(), slices.data(), sizeof(SliceDesc) * ns, cudaMemcpyHostToDevice, h.st));
    NNPP_CUDA(cudaMemcpyAsync(dpre.get(), pre.data(), sizeof(int) * 18 * ns, cudaMemcpyHostToDevice, h.st));
    const int sb = std::max(1, std::min((int)((ns * 32 + 255) / 256), 152 * 32));
    k_slice_windows<<<sb, 256, 0, h.st>>>((int)ns, dsl.get(), dpre.get(), L.row.get(), h.slot16.get(), dlohi.get());
    NNPP_CUDA(cudaGetLastError());
    std::vector<int> lohi(18 * ns);
    NNPP_CUDA(cudaMemcpyAsync(lohi.data(), dlohi.get(), sizeof(int) * 18 * ns, cudaMemcpyDeviceToHost, h.st));
    NNPP_CUDA(cudaStreamSynchronize(h.st));
    // window rows: [lo, hi) rounded out to multiples of 4 nodes (16-byte bulk copies); the
    // codes' 12-bit offsets must reach hi - 1
    for (size_t q = 0; q < ns; ++q) {
      SliceDesc& d = slices[q];
      int acc = 0;
      for (int r = 0; r < 9; ++r) {
        const int lo = lohi[18 * q + r], hi = lohi[18 * q + 9 + r];
        if (hi <= lo) {
          d.lo[r] = 0;
          d.wlen[r] = 0;
        } else {
          d.lo[r] = lo & ~3;
          d.wlen[r] = (hi - d.lo[r] + 3) & ~3;
          if (hi - 1 - d.lo[r] > 4095) return set_error(NNPP_ERR_UNSUPPORTED, "tiles: slice window row wider than 4096 nodes");
        }
        d.woff[r] = acc;
        acc += d.wlen[r];
      }
      d.wtotal = acc;
      for (int r = 0; r < 9; ++r) d.gbase[r] = acc <= 4096 ? d.lo[r] - d.woff[r] : d.lo[r];
      fit = fit && acc <= kWinCap;
    }
    NNPP_CUDA(cudaMemcpyAsync(dsl.get(), slices.data(), sizeof(SliceDesc) * ns, cudaMemcpyHostToDevice, h.st));
    k_sell_fill<<<sb, 256, 0, h.st>>>((int)ns, dsl.get(), dpre.get(), L.row.get(), h.slot16.get(), L.w32.get(),
                                      L.wlo32.get(), h.sell.get(), h.sell_lo.get());
    NNPP_CUDA(cudaGetLastError());
    NNPP_CUDA(cudaStreamSynchronize(h.st));
  }
  *windows_fit = fit;
  gslices.insert(gslices.end(), slices.begin(), slices.end());
  *halo_max = hm;
  *bond_max = bm;
  h.tiles_T = T;
  return NNPP_OK;
}

// Window rows of a slice from the node ranges its bonds reach: [lo, hi) rounded out to
// multiples of 4 nodes (16-byte copies), the codes' 12-bit offsets reaching hi - 1.
static nnpp_status finish_windows(SliceDesc& d, const int* lohi, bool* fit) {
  int acc = 0;
  for (int r = 0; r < 9; ++r) {
    const int lo = lohi[r], hi = lohi[9 + r];
    if (hi <= lo) {
      d.lo[r] = 0;
      d.wlen[r] = 0;
    } else {
      d.lo[r] = lo & ~3;
      d.wlen[r] = (hi - d.lo[r] + 3) & ~3;
      if (hi - 1 - d.lo[r] > 4095) return set_error(NNPP_ERR_UNSUPPORTED, "slice window row wider than 4096 nodes");
    }
    d.woff[r] = acc;
    acc += d.wlen[r];
  }
  d.wtotal = acc;
  for (int r = 0; r < 9; ++r) d.gbase[r] = acc <= 4096 ? d.lo[r] - d.woff[r] : d.lo[r];
  *fit = *fit && acc <= kWinCap;
  return NNPP_OK;
}

nnpp_status build_cg_slices(Handle& h, std::vector<SliceDesc>& gcs, int inst, bool* windows_fit) {
  constexpr unsigned char kPhiDir = 1u << S;
  const Layout& L = h.lay;
  const int N = h.N;
  const int nb0 = L.nb[0], nb1 = L.nb[1], nb2 = L.nb[2];
  if (nb1 > 0xffff || nb2 > 0x7fff) return set_error(NNPP_ERR_UNSUPPORTED, "CG slices: too many bin rows");
  std::vector<int> bs(L.nbins + 1), rows(N + 1);
  std::vector<unsigned char> dm(N);
  NNPP_CUDA(cudaMemcpyAsync(bs.data(), L.bin_start.get(), sizeof(int) * (L.nbins + 1), cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaMemcpyAsync(rows.data(), L.row.get(), sizeof(int) * (N + 1), cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaMemcpyAsync(dm.data(), h.dirmask.get(), (size_t)N, cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  std::vector<int> xrow(N, 0), pos(N, -1), slots;
  std::vector<SliceDesc> cs;
  long long coff = 0;
  std::vector<int> rr, rbx;
  for (int bz = 0; bz < nb2; ++bz)
    for (int by = 0; by < nb1; ++by) {
      const int b0 = nb0 * (by + nb1 * bz);
      const int tag = by | (bz << 16);
      // the row's nodes without a potential Dirichlet value with their bins, in order; a
      // slice takes up to 32 of them from at most two adjacent bins, so that its windows stay
      // a few bins wide where Dirichlet nodes interrupt the row
      rr.clear();
      rbx.clear();
      for (int bx = 0; bx < nb0; ++bx)
        for (int a = bs[b0 + bx]; a < bs[b0 + bx + 1]; ++a) {
          xrow[a] = tag;
          if (!(dm[a] & kPhiDir)) {
            rr.push_back(a);
            rbx.push_back(bx);
          }
        }
      for (size_t i = 0; i < rr.size();) {
        size_t e = i + 1;
        while (e < rr.size() && e - i < 32 && rbx[e] <= rbx[i] + 1) ++e;
        SliceDesc d;
        std::memset(&d, 0, sizeof(d));
        d.inst = inst;
        d.tile = tag;
        d.row0 = (int)slots.size();
        d.nrows = (int)(e - i);
        d.off = (int)coff;
        for (int l = 0; l < 32; ++l) {
          const int a = i + l < e ? rr[i + l] : -1;
          slots.push_back(a);
          if (a >= 0) {
            pos[a] = d.row0 + l;
            d.width = std::max(d.width, rows[a + 1] - rows[a]);
          }
        }
        coff += 32LL * d.width;
        if (coff > 0x7fffffffLL) return set_error(NNPP_ERR_UNSUPPORTED, "CG operator above 2^31 entries");
        cs.push_back(d);
        i = e;
      }
    }
  const size_t ns = cs.size(), nslot = std::max<size_t>(slots.size(), 1);
  if (!h.xrow.alloc(N) || !h.cg_pos.alloc(N) || !h.cg_rows.alloc(nslot) ||
      !h.cg_width.alloc(std::max<size_t>(ns, 1)) || !h.sell_cg.alloc((size_t)(coff / 32) * 48 + 48) ||
      !h.sell_cg_lo.alloc((size_t)(coff / 32) * 32 + 32))
    return set_error(NNPP_ERR_NOMEM, "CG operator");
  NNPP_CUDA(cudaMemcpyAsync(h.xrow.get(), xrow.data(), sizeof(int) * N, cudaMemcpyHostToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(h.cg_pos.get(), pos.data(), sizeof(int) * N, cudaMemcpyHostToDevice, h.st));
  if (!slots.empty())
    NNPP_CUDA(cudaMemcpyAsync(h.cg_rows.get(), slots.data(), sizeof(int) * slots.size(), cudaMemcpyHostToDevice, h.st));
  // filled by the next prep, which forms the rows whenever the unknowns change (every
  // slice empty until then)
  NNPP_CUDA(cudaMemsetAsync(h.cg_width.get(), 0, h.cg_width.bytes(), h.st));
  NNPP_CUDA(cudaMemsetAsync(h.sell_cg.get(), 0, h.sell_cg.bytes(), h.st));
  NNPP_CUDA(cudaMemsetAsync(h.sell_cg_lo.get(), 0, h.sell_cg_lo.bytes(), h.st));
  NNPP_CUDA(cudaMemsetAsync(&h.dstate.get()->op_valid, 0, sizeof(int), h.st));
  bool fit = true;
  if (ns) {
    DBuf<SliceDesc> dsl;
    DBuf<int> dlohi;
    if (!dsl.alloc(ns) || !dlohi.alloc(18 * ns)) return set_error(NNPP_ERR_NOMEM, "CG operator");
    NNPP_CUDA(cudaMemcpyAsync(dsl.get(), cs.data(), sizeof(SliceDesc) * ns, cudaMemcpyHostToDevice, h.st));
    const int sb = std::max(1, std::min((int)((ns * 32 + 255) / 256), 152 * 32));
    k_cg_windows<<<sb, 256, 0, h.st>>>((int)ns, dsl.get(), h.cg_rows.get(), L.row.get(), L.col.get(),
                                       h.dirmask.get(), h.xrow.get(), dlohi.get());
    NNPP_CUDA(cudaGetLastError());
    std::vector<int> lohi(18 * ns);
    NNPP_CUDA(cudaMemcpyAsync(lohi.data(), dlohi.get(), sizeof(int) * 18 * ns, cudaMemcpyDeviceToHost, h.st));
    NNPP_CUDA(cudaStreamSynchronize(h.st));
    for (size_t q = 0; q < ns; ++q) NNPP_TRY(finish_windows(cs[q], lohi.data() + 18 * q, &fit));
  }
  *windows_fit = fit;
  gcs.insert(gcs.end(), cs.begin(), cs.end());
  return NNPP_OK;
}

nnpp_status build_halo_op(Handle& h, int T, const std::vector<TileDesc>& tiles, int tile0,
                          std::vector<HTile>& htiles, int* code_max16, int* quad_max, bool* ok) {
  const Layout& L = h.lay;
  const int N = h.N;
  const int ntile = (int)tiles.size() - tile0;
  *ok = false;
  *code_max16 = 0;
  *quad_max = 0;
  h.halo_op_ok = false;
  HTile none = {0, 0, 0, 0, 0, 0, 0, T};
  // the weights are recomputed as beta / xi^3: kernel exponent s = 0 only; the padding slot
  // of a tile is its halo size, which must fit 16 bits
  bool fits = h.p.s_phi == 0.0;
  for (int t = tile0; t < (int)tiles.size() && fits; ++t) fits = tiles[t].halo < 65535;
  if (!fits) {
    htiles.insert(htiles.end(), ntile, none);
    return NNPP_OK;
  }
  DBuf<int> ddeg;
  if (!ddeg.alloc(N)) return set_error(NNPP_ERR_NOMEM, "halo operator degrees");
  const int blocks = std::max(1, std::min((N + 255) / 256, 152 * 16));
  k_omega_degree<<<blocks, 256, 0, h.st>>>(N, L.row.get(), L.col.get(), h.dirmask.get(), ddeg.get());
  NNPP_CUDA(cudaGetLastError());
  std::vector<int> deg(N), perm(N), bs(L.nbins + 1);
  NNPP_CUDA(cudaMemcpyAsync(deg.data(), ddeg.get(), sizeof(int) * N, cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaMemcpyAsync(perm.data(), L.perm.get(), sizeof(int) * N, cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaMemcpyAsync(bs.data(), L.bin_start.get(), sizeof(int) * (L.nbins + 1), cudaMemcpyDeviceToHost,
                            h.st));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  std::vector<HQuad> quads;
  long long total16 = 0;
  int cmax = 0;
  std::vector<int> rows;
  for (int t = tile0; t < (int)tiles.size(); ++t) {
    const TileDesc& td = tiles[t];
    HTile ht;
    ht.q0 = (int)quads.size();
    ht.cstart16 = (int)total16;
    // bin of the first own node: bins are counting-sorted, so the last bin starting at or
    // before it
    const int b = (int)(std::upper_bound(bs.begin(), bs.end(), td.own_begin) - bs.begin()) - 1;
    ht.by = (b / L.nb[0]) % L.nb[1];
    ht.bz = b / (L.nb[0] * L.nb[1]);
    ht.bx0 = ((b % L.nb[0]) / T) * T;
    ht.T = T;
    rows.clear();
    for (int a = td.own_begin; a < td.own_end; ++a)
      if (deg[a] >= 0) rows.push_back(a);
    // rows of liquid nodes first, longest first (quads of similar length, little padding);
    // nodes solid at the start last, so that slices of solid rows are skipped whole
    std::stable_sort(rows.begin(), rows.end(), [&](int x, int y) {
      const int sx = h.h_phase0[perm[x]] != 0, sy = h.h_phase0[perm[y]] != 0;
      if (sx != sy) return sx < sy;
      return deg[x] > deg[y];
    });
    int coff = 0;
    for (size_t i = 0; i < rows.size(); i += 4) {
      HQuad q;
      int mx = 0;
      for (int g = 0; g < 4; ++g) {
        q.rows[g] = i + g < rows.size() ? rows[i + g] : -1;
        if (q.rows[g] >= 0) mx = std::max(mx, deg[q.rows[g]]);
      }
      q.npass = (mx + 7) / 8;
      q.coff_rel = coff;
      q.coff_abs = (int)(8 * total16) + coff;
      q.padcode = td.halo;
      coff += 32 * q.npass;
      quads.push_back(q);
    }
    ht.nq = (int)quads.size() - ht.q0;
    *quad_max = std::max(*quad_max, ht.nq);
    ht.clen16 = (coff + 7) / 8;
    total16 += ht.clen16;
    if (8 * total16 > 0x7fffffffLL) return set_error(NNPP_ERR_UNSUPPORTED, "halo operator above 2^31 codes");
    cmax = std::max(cmax, ht.clen16);
    htiles.push_back(ht);
  }
  if (!h.hquad.alloc(std::max<size_t>(quads.size(), 1)) || !h.hcode.alloc((size_t)total16 * 8 + 8))
    return set_error(NNPP_ERR_NOMEM, "halo operator");
  NNPP_CUDA(cudaMemsetAsync(h.hcode.get(), 0, ((size_t)total16 * 8 + 8) * sizeof(unsigned short), h.st));
  if (!quads.empty()) {
    NNPP_CUDA(cudaMemcpyAsync(h.hquad.get(), quads.data(), sizeof(HQuad) * quads.size(), cudaMemcpyHostToDevice,
                              h.st));
    const int qb = std::max(1, std::min((int)((4 * quads.size() + 255) / 256), 152 * 16));
    k_fill_hcode<<<qb, 256, 0, h.st>>>((int)quads.size(), h.hquad.get(), L.row.get(), L.col.get(),
                                       h.slot16.get(), h.dirmask.get(), h.hcode.get());
    NNPP_CUDA(cudaGetLastError());
  }
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  *code_max16 = cmax;
  *ok = true;
  h.halo_op_ok = true;
  return NNPP_OK;
}

}  // namespace nnpp
