// emd_gb300: ExaMiniMD's command-line program (main.cpp:48-72) on the GB300
// modules.  Same flags and deck subset as ExaMiniMD.
#include <cstdio>

#include "emd_host.h"

int main(int argc, char* argv[]) {
  try {
    emdhost::ExaMiniMD examinimd;
    examinimd.init(argc, argv);
    examinimd.run(examinimd.input->nsteps);
    examinimd.shutdown();
  } catch (const std::exception& e) {
    fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
