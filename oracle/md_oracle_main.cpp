// ORACLE — test infrastructure only.  `md_oracle <name> [threads]` runs the
// restated reference MD loop (orc_md_run) on <name>.mpd.
#include <cstdlib>
#include <iostream>

#include "smd_oracle.h"

int main(int argc, char* argv[]) {
  if (argc < 2) {
    std::cerr << "usage: " << argv[0] << " name [threads]\n";
    return 0;
  }
  const int threads = argc > 2 ? std::atoi(argv[2]) : 1;
  return orc_md_run(argv[1], threads);
}
