// app.cuh -- drop-in for the reference's include/app.cuh: the gflags the
// samples read (same names and defaults, include/app.cuh:11-31) and
// Skeleton<App>, which parses the command line and runs App::Single() or
// App::Multi() by --ngpu (:33-43).  Two flags are added for the memory
// policy of graph_loader: --mem (device | managed) and --budget.
#ifndef GRUS_MGG_APP_CUH
#define GRUS_MGG_APP_CUH

#include <gflags/gflags.h>

#include <sstream>
#include <string>

#include "common.cuh"
#include "frontier.cuh"
#include "graph.cuh"

DEFINE_string(file, "", "path to task file");
DEFINE_bool(v, false, "verbose results");
DEFINE_bool(pull, false, "use pull-style execution");

DEFINE_int32(device, 0, "GPU ID");
DEFINE_string(input, "", "graph file");
DEFINE_string(output, "", "output result file");

DEFINE_int32(src, 0, "app src");
DEFINE_int32(ngpu, 1, "GPU number, 1 for single-GPU version ");

DEFINE_double(wl_th, 0.5, "wl switch threshold");
DEFINE_bool(pf, false, "use UM prefetch");
DEFINE_bool(ab, false, "use UM hint: AccessedBy");
DEFINE_bool(rm, false, "use UM hint: ReadMostly");
DEFINE_bool(pl, false, "use UM hint: PreferredLocation");
DEFINE_bool(opt, true, "use opt UM policy");

DEFINE_string(mem, "device", "graph memory: device (HBM) or managed");
DEFINE_double(budget, 0, "managed mode device budget: <=1 fraction of CSR bytes, >1 bytes");

template <typename App>
struct Skeleton {
  int operator()(int argc, char **argv) {
    gflags::ParseCommandLineFlags(&argc, &argv, true);
    if (FLAGS_ngpu == 1)
      App::Single();
    else
      App::Multi();
    return 0;
  }
};
#endif
