// Shared-memory plan of the descriptor kernel (host code only; no GPU): prints, for the
// configurations the benchmarks run, the dynamic shared memory per CTA and how many CTAs of it
// fit on one SM, so tests/test_smem_plan.py can hold the kernel to two resident CTAs per SM in
// FP32 (registers allow two; a CTA fewer costs about a third of the kernel's speed).
#include <cstdio>
#include <cstdlib>

#include "../mld_gb300/csrc/bispectrum.cu"

using namespace mld;

namespace {
constexpr size_t kOptin = 227 * 1024;  // opt-in shared memory per CTA
constexpr size_t kPerSm = 228 * 1024;  // shared memory per SM (1 KB of it reserved per CTA)

int ctas(size_t bytes) { return bytes > kOptin ? 0 : (int)(kPerSm / (bytes + 1024)); }
}  // namespace

int main(int argc, char** argv) {
  const double jm = argc > 1 ? std::atof(argv[1]) : 4.0;
  Bso4Tables t;
  std::string err;
  if (!build_bso4_tables(jm, &t, &err)) {
    std::printf("FAIL %s\n", err.c_str());
    return 1;
  }
  DevTables d{};
  fill_dev_tables(t, &d, [](const auto&, auto**) { return cudaSuccess; });
  for (int eb : {4, 8})
    for (int nch : {1, 2, 3}) {
      const size_t ys = smem_plan(d, nch, eb, true).total, yg = smem_plan(d, nch, eb, false).total;
      // as the launch does: Y in shared memory unless that costs a resident CTA (or does not fit)
      const bool shared_y = ctas(ys) >= ctas(yg) && ctas(ys) > 0;
      const size_t s16 = smem_plan(d, nch, eb, shared_y, 16).total;
      int g1 = 16;
      size_t plan = s16;
      for (int g : {4, 6, 8}) {
        const size_t sg = smem_plan(d, nch, eb, shared_y, g).total;
        if (sg <= kOptin && ctas(sg) >= ctas(s16)) {
          g1 = g;
          plan = sg;
          break;
        }
      }
      int cap = 0;
      for (int c = 128; c > 0; c -= 8) {
        const size_t sc = smem_plan(d, nch, eb, shared_y, g1, c).total;
        if (sc <= kOptin && ctas(sc) >= ctas(plan)) {
          cap = c;
          plan = sc;
          break;
        }
      }
      std::printf("eb=%d nch=%d y=%s g1=%d geo_cap=%d bytes=%zu ctas=%d\n", eb, nch, shared_y ? "shared" : "global", g1,
                  cap, plan, ctas(plan));
    }
  return 0;
}
