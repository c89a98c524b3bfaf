// rl_main.cpp -- RADlite_gpu: the drop-in executable. Run in (or given) a RADLite working
// directory; reads the same input files and writes linespectrum_<mol>.dat and
// radlite.success like the reference executable (main.F:26-71). Exit code 0 on success,
// 13 with a message on failure (the reference's `stop 13`).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include "../../include/rlgpu.h"

// `RADlite_gpu --manifest FILE` renders every directory listed in FILE as one batch.
int main(int argc, char** argv) {
  const bool manifest = argc > 2 && std::strcmp(argv[1], "--manifest") == 0;
  const char* dir = argc > 1 ? argv[1] : ".";
  const char* dev = std::getenv("RLGPU_DEVICE");
  rl_stats st;
  const int rc = manifest ? rl_run_manifest(argv[2], dev ? std::atoi(dev) : 0, &st)
                          : rl_run_dir(dir, dev ? std::atoi(dev) : 0, &st);
  if (rc != 0) {
    char msg[1024];
    rl_last_error(nullptr, msg, sizeof msg);
    std::fprintf(stderr, "RADlite_gpu: %s\n", msg);
    return 13;
  }
  std::printf("RADlite_gpu: %d line(s), %d rays x %d channels, walk %.3f ms, geometry %.3f ms\n", st.nlines, st.nrays,
              st.nfr, st.walk_ms, st.geometry_ms);
  return 0;
}
