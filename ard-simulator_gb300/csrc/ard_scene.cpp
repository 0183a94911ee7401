// Host-side scene construction: the reference's object model and setup rules
// (Partition / Boundary / SoundSource / Recorder and the Simulation
// constructor), flattened into the ard_scene description the GPU engine
// takes.  No GPU code here.
//
// Reference behaviour reproduced (paths in ARD-simulator-190113/):
//   Boundary::FindBoundary ........ boundary.cpp:289-334
//   Partition::AddBoundary ........ partition.cpp:96-143 (free-border maps)
//   Simulation::Simulation ........ simulation.cpp:14-294
//       pairwise interfaces (i < j), source attachment (half-open boxes),
//       per air partition: left, right, top, bottom PML runs on z-slice 0
//       of the free-border maps, then front and back PMLs, each followed by
//       its interface; PML runs keep the reference's end-of-row rule (a run
//       whose first non-free cell is the last index extends over it; a run
//       that starts at the last index makes no PML).
//   Recorder::FindPartition ....... recorder.cpp:26-38 (5-cell margin)
//   ImportPartitions / ImportSources / ImportRecorders: integer metres / dh
//       in float, truncated (partition.cpp:151-176, sound_source.cpp:24-48,
//       recorder.cpp:67-89)
//   GaussianSource::SampleValue ... gaussian_source.cpp:16-20
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include "ard_gb300.h"

struct ard_scene_buf {
  ard_scene scene;
  std::vector<ard_partition> parts;
  std::vector<ard_boundary> bounds;
  std::vector<ard_point> sources;
  std::vector<ard_point> recorders;
};

namespace {

thread_local std::string g_scene_error;

int fail(const std::string& msg) {
  g_scene_error = msg;
  return ARD_ERR_INVALID;
}

// One partition while the scene is being assembled: the descriptor plus the
// free-border maps an air partition carries ([depth][height] for left/right,
// [depth][width] for top/bottom).
struct Part {
  ard_partition desc;
  std::vector<std::vector<char>> left, right, top, bottom;
  int xs() const { return desc.x_start; }
  int ys() const { return desc.y_start; }
  int zs() const { return desc.z_start; }
  int xe() const { return desc.x_start + desc.width; }
  int ye() const { return desc.y_start + desc.height; }
  int ze() const { return desc.z_start + desc.depth; }
};

Part make_air(const int32_t* b) {
  Part p{};
  p.desc.kind = ARD_PART_DCT;
  p.desc.pml_type = -1;
  p.desc.x_start = b[0]; p.desc.y_start = b[1]; p.desc.z_start = b[2];
  p.desc.width = b[3]; p.desc.height = b[4]; p.desc.depth = b[5];
  p.left.assign(b[5], std::vector<char>(b[4], 1));
  p.right.assign(b[5], std::vector<char>(b[4], 1));
  p.top.assign(b[5], std::vector<char>(b[3], 1));
  p.bottom.assign(b[5], std::vector<char>(b[3], 1));
  return p;
}

Part make_pml(int type, int x, int y, int z, int w, int h, int d) {
  Part p{};
  p.desc.kind = ARD_PART_PML;
  p.desc.pml_type = type;
  p.desc.x_start = x; p.desc.y_start = y; p.desc.z_start = z;
  p.desc.width = w; p.desc.height = h; p.desc.depth = d;
  return p;
}

// Interface between a and b if they share an x or y face; z range from a.
bool find_boundary(const std::vector<Part>& parts, int ia, int ib, float absorp, ard_boundary* out) {
  const Part& a = parts[ia];
  const Part& b = parts[ib];
  const int x_ov = std::min(a.xe(), b.xe()) - std::max(a.xs(), b.xs());
  const int y_ov = std::min(a.ye(), b.ye()) - std::max(a.ys(), b.ys());
  const int zs = a.zs(), ze = a.zs() + a.desc.depth;
  ard_boundary r{};
  r.a = ia; r.b = ib; r.absorption = absorp; r.z_start = zs; r.z_end = ze;
  if (x_ov == 0 && y_ov > 0) {
    r.type = ARD_BOUNDARY_X;
    r.x_start = (a.xe() == b.xs()) ? a.xe() - 3 : b.xe() - 3;
    r.x_end = r.x_start + 6;
    r.y_start = a.ys() + std::max(0, b.ys() - a.ys());
    r.y_end = r.y_start + y_ov;
    *out = r;
    return true;
  }
  if (y_ov == 0 && x_ov > 0) {
    r.type = ARD_BOUNDARY_Y;
    r.x_start = a.xs() + std::max(0, b.xs() - a.xs());
    r.x_end = r.x_start + x_ov;
    r.y_start = (a.ye() == b.ys()) ? a.ye() - 3 : b.ye() - 3;
    r.y_end = r.y_start + 6;
    *out = r;
    return true;
  }
  return false;
}

void add_boundary(Part& p, const ard_boundary& b) {
  if (b.type == ARD_BOUNDARY_X) {
    auto& map = (b.x_start < p.xs() && b.x_end > p.xs()) ? p.left : p.right;
    for (int i = 0; i < p.desc.depth; ++i)
      for (int j = b.y_start; j < b.y_end; ++j) map[i][j - p.ys()] = 0;
  } else if (b.type == ARD_BOUNDARY_Y) {
    auto& map = (b.y_start < p.ys() && b.y_end > p.ys()) ? p.top : p.bottom;
    for (int i = 0; i < p.desc.depth; ++i)
      for (int j = b.x_start; j < b.x_end; ++j) map[i][j - p.xs()] = 0;
  }
}

// Free runs of one face row, with the reference's end-of-row handling.
std::vector<std::pair<int, int>> pml_runs(const std::vector<char>& free_row) {
  std::vector<std::pair<int, int>> runs;
  const int n = (int)free_row.size();
  int start = 0, end = 0;
  bool started = false;
  for (int i = 0; i < n; ++i) {
    if (started) {
      ++end;
      if (free_row[i] && i != n - 1) continue;
      if (start != end) {
        if (i != n - 1) --end;
        runs.emplace_back(start, end - start + 1);
        started = false;
      }
    } else if (free_row[i]) {
      start = end = i;
      started = true;
    }
  }
  return runs;
}

bool boxes_overlap(const Part& a, const Part& b) {
  return a.xs() < b.xe() && b.xs() < a.xe() && a.ys() < b.ye() && b.ys() < a.ye() &&
         a.zs() < b.ze() && b.zs() < a.ze();
}

}  // namespace

extern "C" int ard_scene_build(const ard_scene_params* params, int32_t n_air, const int32_t* air_boxes,
                               int32_t n_sources, const int32_t* src_cells, int32_t n_recorders,
                               const int32_t* rec_cells, ard_scene_buf** out) {
  if (!params || !out || n_air < 1 || !air_boxes) return fail("ard_scene_build: need params, output and >= 1 air partition");
  if (n_sources < 0 || n_recorders < 0 || (n_sources && !src_cells) || (n_recorders && !rec_cells))
    return fail("ard_scene_build: bad source/recorder arrays");
  if (!(params->dh > 0) || !(params->dt > 0) || !(params->c0 > 0))
    return fail("ard_scene_build: dh, dt and c0 must be positive");
  if (params->pml_layers < 4)
    return fail("ard_scene_build: pml_layers must be >= 4 (the reference's interface orientation test, "
                "boundary.cpp:32,80,128, misreads thinner PMLs)");
  std::vector<Part> parts;
  parts.reserve((size_t)n_air * 8);
  for (int i = 0; i < n_air; ++i) {
    const int32_t* b = air_boxes + 6 * i;
    if (b[3] < 6 || b[4] < 6 || b[5] < 6)
      return fail("ard_scene_build: air partition " + std::to_string(i) +
                  " has an extent below 6 cells (interface strips are 3 cells on each side)");
    parts.push_back(make_air(b));
  }
  for (int i = 0; i < n_air; ++i)
    for (int j = i + 1; j < n_air; ++j)
      if (boxes_overlap(parts[i], parts[j]))
        return fail("ard_scene_build: air partitions " + std::to_string(i) + " and " + std::to_string(j) + " overlap");

  std::vector<ard_boundary> bounds;
  for (int i = 0; i < n_air; ++i)
    for (int j = i + 1; j < n_air; ++j) {
      ard_boundary b;
      if (find_boundary(parts, i, j, 1.0f, &b)) {
        bounds.push_back(b);
        add_boundary(parts[i], b);
        add_boundary(parts[j], b);
      }
    }

  std::vector<ard_point> sources((size_t)n_sources);
  for (int s = 0; s < n_sources; ++s) {
    ard_point& q = sources[s];
    q.x = src_cells[3 * s]; q.y = src_cells[3 * s + 1]; q.z = src_cells[3 * s + 2];
    q.partition = -1;
    for (int i = 0; i < n_air; ++i) {
      const Part& p = parts[i];
      if (q.x >= p.xs() && q.x < p.xe() && q.y >= p.ys() && q.y < p.ye() && q.z >= p.zs() && q.z < p.ze()) {
        q.partition = i;
        break;
      }
    }
  }

  const int L = params->pml_layers;
  const float absorp = params->absorption;
  for (int c = 0; c < n_air; ++c) {
    // parts may grow; copy what the loop needs
    const int xs = parts[c].xs(), ys = parts[c].ys(), zs = parts[c].zs();
    const int xe = parts[c].xe(), ye = parts[c].ye(), ze = parts[c].ze();
    const int w = parts[c].desc.width, h = parts[c].desc.height, d = parts[c].desc.depth;
    const auto left = parts[c].left[0], right = parts[c].right[0];
    const auto top = parts[c].top[0], bottom = parts[c].bottom[0];
    auto add_side = [&](Part pml) {
      parts.push_back(pml);
      ard_boundary b;
      if (!find_boundary(parts, (int)parts.size() - 1, c, absorp, &b)) return false;
      bounds.push_back(b);
      return true;
    };
    for (auto r : pml_runs(left))
      if (!add_side(make_pml(ARD_PML_LEFT, xs - L, ys + r.first, zs, L, r.second, d))) return fail("internal: left PML without interface");
    for (auto r : pml_runs(right))
      if (!add_side(make_pml(ARD_PML_RIGHT, xe, ys + r.first, zs, L, r.second, d))) return fail("internal: right PML without interface");
    for (auto r : pml_runs(top))
      if (!add_side(make_pml(ARD_PML_TOP, xs + r.first, ys - L, zs, r.second, L, d))) return fail("internal: top PML without interface");
    for (auto r : pml_runs(bottom))
      if (!add_side(make_pml(ARD_PML_BOTTOM, xs + r.first, ye, zs, r.second, L, d))) return fail("internal: bottom PML without interface");
    for (int back = 0; back < 2; ++back) {
      parts.push_back(make_pml(back ? ARD_PML_BACK : ARD_PML_FRONT, xs, ys, back ? ze : zs - L, w, h, L));
      ard_boundary b{};
      b.type = ARD_BOUNDARY_Z;
      b.a = (int)parts.size() - 1;
      b.b = c;
      b.x_start = xs; b.x_end = xe; b.y_start = ys; b.y_end = ye;
      b.z_start = (back ? ze : zs) - 3;
      b.z_end = (back ? ze : zs) + 3;
      b.absorption = absorp;
      bounds.push_back(b);
    }
  }

  std::vector<ard_point> recorders((size_t)n_recorders);
  for (int r = 0; r < n_recorders; ++r) {
    ard_point& q = recorders[r];
    q.x = rec_cells[3 * r]; q.y = rec_cells[3 * r + 1]; q.z = rec_cells[3 * r + 2];
    q.partition = -1;
    for (int i = 0; i < n_air; ++i) {
      const Part& p = parts[i];
      if (p.xs() < q.x - 5 && p.xe() > q.x + 4 && p.ys() < q.y - 5 && p.ye() > q.y + 4 &&
          p.zs() < q.z - 5 && p.ze() > q.z + 4) {
        q.partition = i;
        break;
      }
    }
    if (q.partition < 0)
      return fail("ard_scene_build: recorder " + std::to_string(r) +
                  " is not inside any air partition with the 5-cell margin Recorder::FindPartition needs");
  }

  auto* buf = new ard_scene_buf();
  for (auto& p : parts) buf->parts.push_back(p.desc);
  buf->bounds = std::move(bounds);
  buf->sources = std::move(sources);
  buf->recorders = std::move(recorders);
  ard_scene& s = buf->scene;
  s.dh = params->dh; s.dt = params->dt; s.c0 = params->c0;
  s.pml_layers = L;
  s.pml_R = params->pml_R > 0 ? params->pml_R : 1e-5f;
  s.modal_damping = params->modal_damping > 0 ? params->modal_damping : 0.999f;
  s.n_partitions = (int32_t)buf->parts.size(); s.partitions = buf->parts.data();
  s.n_boundaries = (int32_t)buf->bounds.size(); s.boundaries = buf->bounds.data();
  s.n_sources = (int32_t)buf->sources.size(); s.sources = buf->sources.data();
  s.n_recorders = (int32_t)buf->recorders.size(); s.recorders = buf->recorders.data();
  *out = buf;
  return ARD_OK;
}

namespace {

// Integer-metre rows of `group` values, each converted as (int)(v / dh) in float.
bool read_metre_rows(const char* path, float dh, int group, std::vector<int32_t>* cells) {
  std::ifstream f(path);
  if (!f) return false;
  std::vector<int> row(group);
  while (f.good()) {
    for (int k = 0; k < group; ++k) f >> row[k];
    if (f.eof() || f.fail()) break;
    for (int k = 0; k < group; ++k) {
      const float v = (float)row[k] / dh;
      cells->push_back((int32_t)v);
    }
  }
  return true;
}

}  // namespace

extern "C" int ard_scene_import(const ard_scene_params* params, const char* partitions_path,
                                const char* sources_path, const char* recorders_path, ard_scene_buf** out) {
  if (!params || !partitions_path || !sources_path) return fail("ard_scene_import: need params and file paths");
  std::vector<int32_t> boxes, srcs, recs;
  if (!read_metre_rows(partitions_path, params->dh, 6, &boxes))
    return fail(std::string("ard_scene_import: cannot read ") + partitions_path);
  if (!read_metre_rows(sources_path, params->dh, 3, &srcs))
    return fail(std::string("ard_scene_import: cannot read ") + sources_path);
  if (recorders_path && !read_metre_rows(recorders_path, params->dh, 3, &recs))
    return fail(std::string("ard_scene_import: cannot read ") + recorders_path);
  return ard_scene_build(params, (int32_t)(boxes.size() / 6), boxes.data(), (int32_t)(srcs.size() / 3),
                         srcs.data(), (int32_t)(recs.size() / 3), recs.data(), out);
}

extern "C" const ard_scene* ard_scene_get(const ard_scene_buf* buf) { return buf ? &buf->scene : nullptr; }

extern "C" void ard_scene_free(ard_scene_buf* buf) { delete buf; }

extern "C" const char* ard_scene_last_error(void) { return g_scene_error.c_str(); }

extern "C" int ard_gaussian_series(float c0, float dt, float dh, int64_t n, float* out) {
  if (n < 0 || (n > 0 && !out)) return fail("ard_gaussian_series: bad output");
  const float pi = (float)M_PI;
  for (int64_t i = 0; i < n; ++i) {
    const float t = (float)i;
    const float arg = powf(pi * ((2 * (c0 * dt / dh) * t) / 6 - 2.0f), 2);
    out[i] = 1e9f * expf(-arg);
  }
  return ARD_OK;
}
