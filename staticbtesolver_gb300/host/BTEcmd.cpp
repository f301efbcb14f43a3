// BTEcmd.cpp -- executable entry point; the tool itself is sbte_main in BTEMain.cpp.
#include "../../include/sbte.h"
int main(int argc, char** argv) { return sbte_main(argc, argv); }
