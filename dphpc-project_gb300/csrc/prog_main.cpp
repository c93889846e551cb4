// Process entry of a program executable: the whole launcher is gpumpi_main().
#include "gpumpi.h"

int main(int argc, char** argv) { return gpumpi_main(argc, argv); }
