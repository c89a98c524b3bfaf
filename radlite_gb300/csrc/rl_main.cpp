// rl_main.cpp -- RADlite_gpu: the drop-in executable. Run in (or given) a RADLite working
// directory; reads the same input files and writes linespectrum_<mol>.dat (command 0) or
// the lineposvel_<mol>_<iline>.dat cubes (command 2) and radlite.success like the
// reference executable (main.F:26-71, 1034-1074). Exit code 0 on success,
// 13 with a message on failure (the reference's `stop 13`).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include "../../include/rlgpu.h"

// `RADlite_gpu --manifest FILE` renders every directory listed in FILE as one batch;
// `RADlite_gpu --save-imcir [dir]` behaves as a reference build with SAVE_IMCIR
// (configure_image.h) and also writes the circular image of every line.
int main(int argc, char** argv) {
  int a = 1, flags = 0;
  if (argc > a && std::strcmp(argv[a], "--save-imcir") == 0) { flags |= RL_RUN_SAVE_IMCIR; a++; }
  const bool manifest = argc > a + 1 && std::strcmp(argv[a], "--manifest") == 0;
  const char* dir = argc > a ? argv[a] : ".";
  const char* dev = std::getenv("RLGPU_DEVICE");
  rl_stats st;
  const int rc = manifest ? rl_run_manifest(argv[a + 1], dev ? std::atoi(dev) : 0, &st)
                          : rl_run_dir_ex(dir, dev ? std::atoi(dev) : 0, flags, &st);
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
