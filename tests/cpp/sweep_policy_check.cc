// Host-only check of the mixed-precision sweep policy (MixedSweeps, cc_ground.cpp): feeds
// residual-norm trajectories to the policy and prints, per sweep, the kind it chose, the
// digits of record sweeps and whether the solve ended.  No CUDA call is made: the policy
// and the anchor bookkeeping it touches are host state of the context.
#include <cstdio>
#include <vector>

#include "cc.h"
#include "pert.h"  // the context owns its perturbations

using namespace ucc;

static const char* kind_name(MixedSweeps::Kind k) {
  return k == MixedSweeps::kSplit ? "split" : k == MixedSweeps::kRecord ? "record" : k == MixedSweeps::kDelta ? "delta"
                                                                                                                 : "fp64";
}

// one line per sweep: kind[:digits] and "done" on the last
static void run(const char* name, double rc, const std::vector<double>& rms) {
  Ctx c;
  ucc_options_default(&c.opt);
  c.opt.precision = UCC_MIXED;
  c.opt.r_convergence = rc;
  MixedSweeps sw(c);
  std::printf("%s:", name);
  for (double r : rms) {
    const MixedSweeps::Kind k = sw.begin();
    const int digits = c.anchors.digits;
    sw.end();
    bool restart = false;
    const bool done = sw.after(r, &restart);
    if (k == MixedSweeps::kRecord)
      std::printf(" record:%d", digits);
    else
      std::printf(" %s", kind_name(k));
    if (done) {
      std::printf(" done");
      break;
    }
  }
  std::printf("\n");
}

int main() {
  // the no=32/nv=320 solve from the MP2 guess (R_CONVERGENCE 1e-10)
  run("mp2", 1e-10,
      {0.43, 0.23, 0.14, 3.4e-3, 3.3e-4, 8e-5, 1.4e-5, 7.4e-6, 4.5e-5, 2.4e-5, 1.5e-5, 2.4e-7, 3.4e-8, 5.2e-9,
       1.5e-9, 3.1e-10, 4.5e-11, 4.5e-11});
  // a good start: one slow split sweep far above the split floor does not hand over
  run("guess", 1e-10, {0.059, 0.0104, 0.0053, 3.0e-4, 6.0e-5, 8.0e-6});
  // two slow split sweeps in a row within three decades of the floor hand over
  run("stall", 1e-10, {0.43, 0.1, 5.0e-3, 4.0e-3, 3.5e-3, 3.0e-3});
  // deltas that stop falling ask for a full-digit anchor
  run("dstall", 1e-10, {0.1, 8e-6, 4e-5, 1e-5, 9e-6, 8.5e-6, 8e-6});
  // a record sweep with fewer digits whose residual is already below R_CONVERGENCE does
  // not end the solve: a 9-digit confirmation follows
  run("early", 1e-7, {0.1, 8e-6, 5e-8, 5e-8});
  return 0;
}
