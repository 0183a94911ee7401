/* ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Headless driver for the reference ARD simulator.  It is linked against the
 * reference's own, unmodified sources (compiled in place by the Makefile in
 * this directory) and replaces only ARD-simulator-190113/main.cpp, which needs
 * Windows, SDL and Vulkan.  Like main.cpp:29-45 it defines the simulation's
 * static parameters, then builds DctPartitions in cell units, attaches
 * sources, constructs Simulation (interface discovery and PML generation run
 * as in the reference) and steps it.
 *
 * Usage: ard_ref <config-file>
 *
 * Modes
 *   reference  calls Simulation::Update() (simulation.cpp:300-421) each step,
 *              visualisation block included, with whatever OMP_NUM_THREADS is.
 *   parity     runs the same per-step work in the order a single thread would:
 *              phase A (source forcing + Partition::Update) in parallel over
 *              partitions, which is order-independent, then phase B
 *              (Boundary::ComputeForcingTerms) serially in list order, which
 *              is what makes overlapping interface writes deterministic.  The
 *              visualisation block only fills a pixel buffer and is skipped.
 *
 * Recorders are sampled after every step at the intended cell (global cell
 * minus the partition origin), in the partition Recorder::FindPartition
 * (recorder.cpp:26-38) would pick.
 */
#include <omp.h>
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <limits>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

/* Reach the members the setup dump needs without editing reference headers:
 * the reference classes rely on class-default private access, so the class
 * key is switched to struct (same type, same layout) and the explicit
 * access labels are opened. */
#define class struct
#define private public
#define protected public
#include "boundary.h"
#include "dct_partition.h"
#include "gaussian_source.h"
#include "partition.h"
#include "pml_partition.h"
#include "simulation.h"
#include "sound_source.h"
#undef class
#undef private
#undef protected

real_t Partition::m_absorption = 1.0f;
real_t Simulation::m_duration = 2.0f;
real_t Simulation::m_dh = 0.1f;
real_t Simulation::m_dt = 1.0f / 8000.0f;
real_t Simulation::m_c0 = 3.435e2f;
int Simulation::m_pml_layers = 5;

namespace {

class SeriesSource : public SoundSource {
 public:
  SeriesSource(int x, int y, int z, std::vector<float> s)
      : SoundSource(x, y, z), series_(std::move(s)) {}
  real_t SampleValue(real_t t) override {
    long i = (long)t;
    return (i >= 0 && i < (long)series_.size()) ? series_[i] : 0.0f;
  }

 private:
  std::vector<float> series_;
};

float read_float(std::istream& in) {
  std::string tok;
  in >> tok;
  return std::strtof(tok.c_str(), nullptr);
}

struct RecorderSpec {
  int x, y, z;
  int part;
};

void die(const std::string& msg) {
  std::fprintf(stderr, "ard_ref: %s\n", msg.c_str());
  std::exit(2);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 2) die("usage: ard_ref <config>");
  std::ifstream cfg(argv[1]);
  if (!cfg) die("cannot open config");

  std::string key, mode = "parity", outdir = ".";
  int steps = 0;
  std::vector<std::vector<int>> part_boxes;
  std::vector<std::shared_ptr<SoundSource>> sources;
  std::vector<RecorderSpec> recorders;
  std::vector<int> field_steps;
  std::vector<std::string> source_lines;

  /* Parameters must be set before any partition or source is constructed
   * (their constructors read Simulation::m_dh etc.), so sources are kept as
   * text until the header has been read. */
  while (cfg >> key) {
    if (key == "dh") Simulation::m_dh = read_float(cfg);
    else if (key == "dt") Simulation::m_dt = read_float(cfg);
    else if (key == "c0") Simulation::m_c0 = read_float(cfg);
    else if (key == "duration") Simulation::m_duration = read_float(cfg);
    else if (key == "absorption") Partition::m_absorption = read_float(cfg);
    else if (key == "pml_layers") cfg >> Simulation::m_pml_layers;
    else if (key == "steps") cfg >> steps;
    else if (key == "mode") cfg >> mode;
    else if (key == "out") cfg >> outdir;
    else if (key == "partitions") {
      int n; cfg >> n;
      for (int i = 0; i < n; ++i) {
        std::vector<int> b(6);
        for (int& v : b) cfg >> v;
        part_boxes.push_back(b);
      }
    } else if (key == "sources") {
      int n; cfg >> n;
      std::string line;
      std::getline(cfg, line);
      for (int i = 0; i < n; ++i) {
        std::getline(cfg, line);
        source_lines.push_back(line);
      }
    } else if (key == "recorders") {
      int n; cfg >> n;
      for (int i = 0; i < n; ++i) {
        RecorderSpec r{};
        cfg >> r.x >> r.y >> r.z;
        r.part = -1;
        recorders.push_back(r);
      }
    } else if (key == "fields") {
      int n; cfg >> n;
      for (int i = 0; i < n; ++i) { int s; cfg >> s; field_steps.push_back(s); }
    } else {
      die("unknown key " + key);
    }
  }

  for (const std::string& line : source_lines) {
    std::istringstream ls(line);
    int x, y, z;
    std::string kind;
    ls >> x >> y >> z >> kind;
    if (kind == "gaussian") {
      sources.push_back(std::make_shared<GaussianSource>(x, y, z));
    } else if (kind == "series") {
      int n; ls >> n;
      std::vector<float> s(n);
      for (int i = 0; i < n; ++i) s[i] = read_float(ls);
      sources.push_back(std::make_shared<SeriesSource>(x, y, z, s));
    } else {
      die("bad source kind " + kind);
    }
  }

  VkGPU gpu{};
  std::vector<std::shared_ptr<Partition>> partitions;
  for (auto& b : part_boxes)
    partitions.push_back(std::make_shared<DctPartition>(b[0], b[1], b[2], b[3], b[4], b[5], &gpu));

  /* Recorder::FindPartition over the air partitions (main.cpp:84-87). */
  for (auto& r : recorders) {
    for (size_t i = 0; i < partitions.size(); ++i) {
      auto& p = partitions[i];
      if (p->x_start_ < r.x - 5 && p->x_end_ > r.x + 4 &&
          p->y_start_ < r.y - 5 && p->y_end_ > r.y + 4 &&
          p->z_start_ < r.z - 5 && p->z_end_ > r.z + 4) {
        r.part = (int)i;
        break;
      }
    }
  }

  auto sim = std::make_shared<Simulation>(partitions, sources);
  auto& parts = sim->m_partitions;
  auto& bounds = sim->m_boundaries;

  mkdir(outdir.c_str(), 0755);
  {
    std::ofstream s(outdir + "/setup.txt");
    auto index_of = [&](const std::shared_ptr<Partition>& p) {
      for (size_t i = 0; i < parts.size(); ++i)
        if (parts[i].get() == p.get()) return (int)i;
      return -1;
    };
    for (size_t i = 0; i < parts.size(); ++i) {
      auto& p = parts[i];
      auto* pml = dynamic_cast<PmlPartition*>(p.get());
      s << "P " << i << " " << (pml ? "PML" : "DCT") << " " << (pml ? (int)pml->type_ : -1) << " "
        << p->x_start_ << " " << p->y_start_ << " " << p->z_start_ << " "
        << p->width_ << " " << p->height_ << " " << p->depth_ << "\n";
    }
    for (size_t i = 0; i < bounds.size(); ++i) {
      auto& b = bounds[i];
      char ab[64];
      std::snprintf(ab, sizeof ab, "%a", (double)b->absorption_);
      s << "B " << i << " " << (int)b->type_ << " " << index_of(b->a_) << " " << index_of(b->b_) << " "
        << b->x_start_ << " " << b->x_end_ << " " << b->y_start_ << " " << b->y_end_ << " "
        << b->z_start_ << " " << b->z_end_ << " " << ab << "\n";
    }
    for (size_t i = 0; i < parts.size(); ++i)
      for (auto& src : parts[i]->sources_) s << "S " << i << " " << src->id_ << "\n";
    for (size_t i = 0; i < recorders.size(); ++i) s << "R " << i << " " << recorders[i].part << "\n";
  }

  /* SoundSource::SampleValue(t) of every source for t < steps, as injected */
  {
    std::FILE* sf = std::fopen((outdir + "/sources.f32").c_str(), "wb");
    for (auto& src : sources)
      for (int t = 0; t < steps; ++t) {
        float v = src->SampleValue((real_t)t);
        std::fwrite(&v, sizeof v, 1, sf);
      }
    std::fclose(sf);
  }

  std::FILE* rec = std::fopen((outdir + "/recorders.f32").c_str(), "wb");
  std::vector<float> sample(recorders.size());

  const double t0 = omp_get_wtime();
  for (int step = 0; step < steps; ++step) {
    if (mode == "reference") {
      sim->Update();
    } else {
      const int n = (int)parts.size();
#pragma omp parallel for schedule(dynamic, 1)
      for (int i = 0; i < n; ++i) {
        parts[i]->ComputeSourceForcingTerms((real_t)step);
        parts[i]->Update();
      }
      for (auto& b : bounds) b->ComputeForcingTerms();
      sim->time_step_++;
    }
    for (size_t r = 0; r < recorders.size(); ++r) {
      const auto& rs = recorders[r];
      if (rs.part < 0) { sample[r] = NAN; continue; }
      auto& p = partitions[rs.part];
      sample[r] = p->get_pressure(rs.x - p->x_start_, rs.y - p->y_start_, rs.z - p->z_start_);
    }
    if (!sample.empty()) std::fwrite(sample.data(), sizeof(float), sample.size(), rec);
    if (std::find(field_steps.begin(), field_steps.end(), step) != field_steps.end()) {
      std::FILE* f = std::fopen((outdir + "/fields_" + std::to_string(step) + ".f32").c_str(), "wb");
      for (auto& p : parts) {
        const long n = (long)p->width_ * p->height_ * p->depth_;
        std::vector<float> pres(n), force(n);
        if (auto* d = dynamic_cast<DctPartition*>(p.get())) {
          std::memcpy(pres.data(), d->m_pressure.m_values, n * sizeof(float));
          std::memcpy(force.data(), d->m_force.m_values, n * sizeof(float));
        } else {
          auto* q = dynamic_cast<PmlPartition*>(p.get());
          std::memcpy(pres.data(), q->p_, n * sizeof(float));
          std::memcpy(force.data(), q->force_, n * sizeof(float));
        }
        std::fwrite(pres.data(), sizeof(float), n, f);
        std::fwrite(force.data(), sizeof(float), n, f);
      }
      std::fclose(f);
    }
  }
  const double t1 = omp_get_wtime();
  std::fclose(rec);

  long air = 0, pml = 0;
  for (auto& p : parts) {
    const long n = (long)p->width_ * p->height_ * p->depth_;
    if (dynamic_cast<DctPartition*>(p.get())) air += n; else pml += n;
  }
  std::printf("{\"seconds\": %.6f, \"steps\": %d, \"threads\": %d, \"air_cells\": %ld, \"pml_cells\": %ld, \"mode\": \"%s\"}\n",
              t1 - t0, steps, omp_get_max_threads(), air, pml, mode.c_str());
  return 0;
}
