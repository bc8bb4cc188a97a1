// rwnmr_gb300 executable: the command-line driver (see app.cpp).
#include "rwnmr_host.h"

int main(int argc, char **argv) { return rwnmr_cli_main(argc, (const char *const *)argv); }
