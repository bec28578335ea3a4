// main.cpp - the `umcx` command-line program (fangq/umcx src/umcx.cpp:868-875) on the GB300 library.
#include "../../include/umcx_host.h"

int main(int argc, char* argv[]) { return umcx_main(argc, argv); }
