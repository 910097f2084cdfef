// `MD <name>`: drop-in for the reference executable (MD.cpp:72-81).
// SMD_PRECISION=plain selects the all-FP64 form; the default is mixed.
#include <cstdlib>
#include <cstring>
#include <iostream>

#include "../../include/softmold_gb300.h"

int main(int argc, char* argv[]) {
  if (argc != 2) {
    std::cerr << "usage: " << argv[0] << " name\n";
    return 0;
  }
  const char* p = std::getenv("SMD_PRECISION");
  const int precision = (p && std::strcmp(p, "plain") == 0) ? SMD_PLAIN_FP64 : SMD_MIXED;
  return smd_md_main(argv[1], precision);
}
