// Host-side helpers shared by the batch plan (batch.cu) and the serving
// queue (queue.cu): the work-list builder of the persistent batch kernel
// (fft_batch.cuh), convolution geometry, and the resident tables.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <deque>
#include <vector>

#include "../../include/tcfft_gb300.h"
#include "fft_batch.cuh"
#include "tables.cuh"

namespace tcfft {

// Registry of the batch kernel (batch.cu): kernel and CTA count per
// precision (0 FP16, 1 split) and direction (0 forward, 1 inverse).
tcfftStatus batch_registry_ready();
const BatchKernel& batch_kernel(int precision_idx, int sign_idx);
int batch_ctas(int precision_idx, int sign_idx);

namespace bh {

inline int ilog2_exact(long long v) {
  if (v <= 0 || (v & (v - 1)) != 0) return -1;
  int l = 0;
  while ((1ll << l) < v) ++l;
  return l;
}

// Four-step split used by the batch kernel: both pass lengths in [2^7, 2^10].
inline int batch_log_n1(int logn) {
  int a = logn / 2;
  if (a < kBatchMinPassLog) a = kBatchMinPassLog;
  if (logn - a > kBatchMaxPassLog) a = logn - kBatchMaxPassLog;
  return a;
}

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// What to put in one launch: 1D transforms (offsets in elements) and
// convolutions with geometry, buffer offsets, spectrum and filter filled in;
// conv_prep[c] != 0 adds the tiles that make convolution c's spectrum.
struct BatchSpec {
  int count = 0;
  const long long* n = nullptr;
  const long long* in_off = nullptr;
  const long long* out_off = nullptr;
  const float* scale = nullptr;  // per transform (not null when count > 0)
  std::vector<BatchConv> convs;
  std::vector<char> conv_prep;
  bool fuse_conv_columns = false;  // FP16: both column FFTs as one item kind (kItemConvMid)
};

struct Built {
  std::vector<long long> line_in, line_out;
  std::vector<BatchItem> items;       // main launch
  std::vector<BatchItem> prep_items;  // filter-spectrum launch
  std::vector<BatchXform> xforms;
  std::vector<BatchConv> convs;       // with workspace offsets
  size_t ws_elems = 0;
  int nctrs = 0;  // dependency counters ([0] is the queue head)
};

// Padded size and output window of a convolution (the rule of
// tcfft_conv2d_plan: the smallest power of two without wrap-around inside
// the output window).
inline bool conv_geometry(const tcfftBatchConv& d, BatchConv& cv) {
  long long need;
  cv.flip = 0;
  if (d.mode == TCFFT_CONV_VALID_CORR) {
    if (d.fy > d.sy || d.fx > d.sx) return false;
    need = std::max(d.sy, d.sx);
    cv.oy = d.sy - d.fy + 1;
    cv.ox = d.sx - d.fx + 1;
    cv.r0 = d.fy - 1;
    cv.c0 = d.fx - 1;
    cv.flip = 1;
  } else if (d.mode == TCFFT_CONV_SAME) {
    if (d.fy % 2 == 0 || d.fx % 2 == 0) return false;
    need = std::max(d.sy + (d.fy - 1) / 2, d.sx + (d.fx - 1) / 2);
    cv.oy = d.sy;
    cv.ox = d.sx;
    cv.r0 = (d.fy - 1) / 2;
    cv.c0 = (d.fx - 1) / 2;
  } else if (d.mode == TCFFT_CONV_FULL) {
    need = std::max(d.sy + d.fy - 1, d.sx + d.fx - 1);
    cv.oy = d.sy + d.fy - 1;
    cv.ox = d.sx + d.fx - 1;
    cv.r0 = 0;
    cv.c0 = 0;
  } else {
    return false;
  }
  int l = kBatchMinConvLog;
  while ((1ll << l) < need) ++l;
  if (l > kBatchMaxConvLog) return false;
  cv.logP = l;
  cv.sy = d.sy;
  cv.sx = d.sx;
  cv.fy = d.fy;
  cv.fx = d.fx;
  return true;
}

inline BatchItem make_item(int kind, int logl, int line0, int obj, float scale) {
  BatchItem it{};
  it.kind = kind;
  it.logl = logl;
  it.line0 = line0;
  it.obj = obj;
  it.scale = scale;
  it.wait_ctr = -1;
  it.signal_ctr = -1;
  return it;
}

// Tiles of one pass over `lines` lines of length 2^logl.
inline void add_tiles(std::vector<BatchItem>& v, int kind, int logl, int lines, int obj, float scale, int wait_ctr,
               int wait_target, int signal_ctr) {
  const int g = kBatchMt * 16 >> logl;
  for (int t = 0; t * g < lines; ++t) {
    BatchItem it = make_item(kind, logl, t * g, obj, scale);
    it.wait_ctr = wait_ctr;
    it.wait_target = wait_target;
    it.signal_ctr = signal_ctr;
    v.push_back(it);
  }
}

inline int tiles_of(int logl, int lines) {
  const int g = kBatchMt * 16 >> logl;
  return (lines + g - 1) / g;
}

// Work list: single-pass 1D transforms grouped by size into tiles of
// G = 8192 / L lines; every multi-stage job (four-step transform,
// convolution) emits its first stage, then each later stage `lag` items after
// the stage before; single-pass tiles are spread evenly in between.
inline Built build_items(const BatchSpec& b, int lag) {
  Built out;
  out.nctrs = 1;  // [0] is the queue head
  std::vector<BatchItem> line_items;
  for (int logl = kBatchMinLineLog; logl <= kBatchMaxLineLog; ++logl) {
    const int G = kBatchMt * 16 >> logl;
    std::vector<int> ids;
    for (int i = 0; i < b.count; ++i)
      if (ilog2_exact(b.n[i]) == logl) ids.push_back(i);
    size_t k = 0;
    while (k < ids.size()) {
      // one scale per tile: split the tile where the scale changes
      size_t end = std::min(ids.size(), k + static_cast<size_t>(G));
      for (size_t j = k + 1; j < end; ++j)
        if (b.scale[ids[j]] != b.scale[ids[k]]) {
          end = j;
          break;
        }
      BatchItem it = make_item(kItemLines, logl, static_cast<int>(out.line_in.size()), 0, b.scale[ids[k]]);
      it.nlines = static_cast<int>(end - k);
      for (size_t j = k; j < end; ++j) {
        out.line_in.push_back(b.in_off[ids[j]]);
        out.line_out.push_back(b.out_off[ids[j]]);
      }
      line_items.push_back(it);
      k = end;
    }
  }
  using Stages = std::vector<std::vector<BatchItem>>;
  std::vector<Stages> jobs;
  for (int i = 0; i < b.count; ++i) {
    const int logn = ilog2_exact(b.n[i]);
    if (logn <= kBatchMaxLineLog) continue;
    BatchXform xf{};
    xf.in_off = b.in_off[i];
    xf.out_off = b.out_off[i];
    xf.ws_off = static_cast<long long>(out.ws_elems);
    xf.logn = logn;
    xf.log_n1 = batch_log_n1(logn);
    xf.log_n2 = logn - xf.log_n1;
    out.ws_elems += static_cast<size_t>(b.n[i]);
    xf.tiles1 = tiles_of(xf.log_n1, 1 << xf.log_n2);
    const int obj = static_cast<int>(out.xforms.size());
    const int ctr = out.nctrs++;
    Stages st(2);
    add_tiles(st[0], kItemP1, xf.log_n1, 1 << xf.log_n2, obj, 1.0f, -1, 0, ctr);
    add_tiles(st[1], kItemP2, xf.log_n2, 1 << xf.log_n1, obj, b.scale[i], ctr, xf.tiles1, -1);
    out.xforms.push_back(xf);
    jobs.push_back(std::move(st));
  }
  for (size_t c = 0; c < b.convs.size(); ++c) {
    BatchConv cv = b.convs[c];
    const int P = 1 << cv.logP;
    const long long rows = std::max({cv.sy, cv.oy, cv.fy});
    cv.x_off = static_cast<long long>(out.ws_elems);
    out.ws_elems += static_cast<size_t>(rows) * P;
    cv.y_off = static_cast<long long>(out.ws_elems);
    if (!b.fuse_conv_columns) out.ws_elems += static_cast<size_t>(P) * P;
    const int obj = static_cast<int>(out.convs.size());
    const float inv_p = 1.0f / static_cast<float>(P);
    if (b.conv_prep[c]) {
      // filter spectrum (a separate launch before the main one)
      const int fc = out.nctrs++;
      add_tiles(out.prep_items, kItemFiltRow, cv.logP, cv.fy, obj, 1.0f, -1, 0, fc);
      add_tiles(out.prep_items, kItemFiltCol, cv.logP, P, obj, 1.0f, fc, tiles_of(cv.logP, cv.fy), -1);
    }
    // the convolution
    Stages st;
    if (b.fuse_conv_columns) {
      const int c1 = out.nctrs++, c2 = out.nctrs++;
      st.resize(3);
      add_tiles(st[0], kItemConvRow, cv.logP, cv.sy, obj, inv_p, -1, 0, c1);
      add_tiles(st[1], kItemConvMid, cv.logP, P, obj, inv_p, c1, tiles_of(cv.logP, cv.sy), c2);
      add_tiles(st[2], kItemConvOut, cv.logP, cv.oy, obj, 1.0f, c2, tiles_of(cv.logP, P), -1);
    } else {
      const int c1 = out.nctrs++, c2 = out.nctrs++, c3 = out.nctrs++;
      st.resize(4);
      add_tiles(st[0], kItemConvRow, cv.logP, cv.sy, obj, inv_p, -1, 0, c1);
      add_tiles(st[1], kItemConvCol, cv.logP, P, obj, inv_p, c1, tiles_of(cv.logP, cv.sy), c2);
      add_tiles(st[2], kItemConvInv, cv.logP, P, obj, 1.0f, c2, tiles_of(cv.logP, P), c3);
      add_tiles(st[3], kItemConvOut, cv.logP, cv.oy, obj, 1.0f, c3, tiles_of(cv.logP, P), -1);
    }
    out.convs.push_back(cv);
    jobs.push_back(std::move(st));
  }
  // merge
  size_t total = line_items.size();
  for (const Stages& j : jobs)
    for (const auto& g : j) total += g.size();
  out.items.reserve(total);
  struct Pending {
    size_t ready;
    size_t job, stage;
  };
  std::deque<Pending> pending;  // ready positions are nondecreasing
  auto emit_stage = [&](size_t job, size_t stage) {
    for (const BatchItem& it : jobs[job][stage]) out.items.push_back(it);
    if (stage + 1 < jobs[job].size()) pending.push_back({out.items.size() + static_cast<size_t>(lag), job, stage + 1});
  };
  auto release = [&](bool all) {
    while (!pending.empty() && (all || pending.front().ready <= out.items.size())) {
      const Pending p = pending.front();
      pending.pop_front();
      emit_stage(p.job, p.stage);
    }
  };
  size_t li = 0;
  const double per_job = jobs.empty() ? 0.0 : static_cast<double>(line_items.size()) / jobs.size();
  double credit = 0.0;
  for (size_t j = 0; j < jobs.size(); ++j) {
    release(false);
    emit_stage(j, 0);
    credit += per_job;
    while (credit >= 1.0 && li < line_items.size()) {
      out.items.push_back(line_items[li++]);
      credit -= 1.0;
      release(false);
    }
  }
  while (li < line_items.size()) {
    out.items.push_back(line_items[li++]);
    release(false);
  }
  while (!pending.empty()) release(true);
  return out;
}


}  // namespace bh
}  // namespace tcfft
