// Host-side check of the fused face transforms' job balancer
// (ard::balance_face_jobs, ard_layout.cu), linked against the built library.
// Built and run by tests/test_face_balancer.py; no GPU is touched.
//
// For job lists of several shapes and wave sizes it checks that the output
// is a list of cluster pairs (a row-split job twice, or two whole jobs, the
// last padded by an empty job), that every (layer pair, slab, output) of the
// input is produced by exactly one pair entry, that splits stop at one wave
// of CTAs, that a list of a wave or more is left whole, that the narrow
// flag follows the slab width and that the return value reports the splits.
#define __host__
#define __device__
#include <cstdio>
#include <map>
#include <tuple>
#include <vector>

#include "ard_device.cuh"

namespace ard {
bool balance_face_jobs(std::vector<Face2DJob>* jobs, int slots);
}

using ard::Face2DJob;

static int failures = 0;
#define CHECK(c, ...)                                  \
  do {                                                 \
    if (!(c)) {                                        \
      std::printf("FAIL %s:%d: ", __FILE__, __LINE__); \
      std::printf(__VA_ARGS__);                        \
      std::printf("\n");                               \
      ++failures;                                      \
    }                                                  \
  } while (0)

// One face of V x U: three layer pairs, slabs of 32 columns (the layout's form).
static void add_face(std::vector<Face2DJob>* jobs, int V, int U, long long base) {
  for (int u0 = 0; u0 < U; u0 += 32)
    for (int n = 0; n < 3; ++n) {
      Face2DJob j{};
      j.in0 = base + n;
      j.in1 = base + 5 - n;
      j.out0 = base + 100 + n;
      j.out1 = base + 200 + n;
      j.V = V;
      j.U = U;
      j.ld = U;
      j.u0 = u0;
      j.ub = U - u0 < 32 ? U - u0 : 32;
      j.which = 0;
      j.scale = 1.0;
      jobs->push_back(j);
    }
}

using Unit = std::tuple<long long, int, long long>;   // (in0, u0, output)

static void check(const std::vector<Face2DJob>& in, int slots, const char* name, int expect_split) {
  std::vector<Face2DJob> out = in;
  const bool split = ard::balance_face_jobs(&out, slots);
  CHECK(out.size() % 2 == 0, "%s: odd entry count %zu", name, out.size());
  std::map<Unit, int> want, got;
  for (const Face2DJob& j : in) {
    want[Unit(j.in0, j.u0, j.out0)] += 1;
    want[Unit(j.in0, j.u0, j.out1)] += 1;
  }
  long long ctas = 0;
  bool any_split = false;
  for (size_t i = 0; i + 1 < out.size(); i += 2) {
    const Face2DJob& a = out[i];
    const Face2DJob& b = out[i + 1];
    if (a.split) {
      any_split = true;
      CHECK(b.split && b.in0 == a.in0 && b.u0 == a.u0 && b.which == a.which && b.V == a.V,
            "%s: pair %zu: a split job must fill both entries", name, i / 2);
      CHECK(a.which != 0, "%s: pair %zu: a split job has one output", name, i / 2);
      CHECK(a.V > 1, "%s: pair %zu: a split job has two rows or more", name, i / 2);
      ctas += 2;
    } else {
      CHECK(!b.split, "%s: pair %zu: a whole job paired with a split one", name, i / 2);
    }
    const int n = a.split ? 1 : 2;
    for (int k = 0; k < n; ++k) {
      const Face2DJob& j = k ? b : a;
      if (j.V == 0) continue;   // the empty pad of the last pair
      if (!a.split) ctas += 1;
      CHECK(j.narrow == (j.ub <= 16 ? 1 : 0), "%s: narrow flag of a %d-column slab", name, j.ub);
      if (j.which != 2) got[Unit(j.in0, j.u0, j.out0)] += 1;
      if (j.which != 1) got[Unit(j.in0, j.u0, j.out1)] += 1;
    }
  }
  CHECK(got == want, "%s: the pairs do not produce every output slab exactly once", name);
  CHECK(split == any_split, "%s: return value %d, split jobs %d", name, (int)split, (int)any_split);
  CHECK((int)any_split == expect_split, "%s: row splits %d, expected %d", name, (int)any_split, expect_split);
  const long long n_in = (long long)in.size();
  if (n_in >= slots) {
    CHECK(ctas == n_in && !any_split, "%s: a list of a wave or more is left whole", name);
  } else {
    // splits add one CTA each and stop once a wave is reached
    CHECK(ctas <= (long long)slots, "%s: %lld CTAs for a wave of %d", name, ctas, slots);
  }
}

int main() {
  {
    std::vector<Face2DJob> jobs;   // one large partition, few jobs: splits down to row halves
    add_face(&jobs, 120, 120, 0);
    add_face(&jobs, 80, 120, 1000);
    add_face(&jobs, 80, 120, 2000);
    check(jobs, 176, "c1-like group", 1);
    check(jobs, 304, "c1-like group, two waves of slots", 1);
    check(jobs, 40, "c1-like group, a wave of 40 CTAs", 0);
  }
  {
    std::vector<Face2DJob> jobs;   // ragged extents and narrow tails
    add_face(&jobs, 1, 4, 0);
    add_face(&jobs, 9, 13, 1000);
    add_face(&jobs, 40, 40, 2000);
    add_face(&jobs, 37, 50, 3000);
    check(jobs, 304, "ragged faces", 1);
    check(jobs, 7, "ragged faces, a short wave", 0);
  }
  {
    std::vector<Face2DJob> jobs;   // many small faces: more jobs than a wave, left whole
    for (int s = 0; s < 120; ++s) add_face(&jobs, 40 + s % 7, 30 + s % 11, 10000LL * s);
    check(jobs, 304, "c2-like batch", 0);
  }
  {
    std::vector<Face2DJob> jobs;   // an odd number of whole jobs: the last pair is padded
    add_face(&jobs, 20, 20, 0);
    check(jobs, 3, "odd whole list", 0);
  }
  if (failures) {
    std::printf("%d failure(s)\n", failures);
    return 1;
  }
  std::printf("face balancer ok\n");
  return 0;
}
