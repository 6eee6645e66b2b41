// cgppd_main.cpp -- the `cgppd` command: same command line and argfile as the
// reference's executable (src/main.cpp), every replica on the GPU engine.
#include <unistd.h>

extern "C" int cgppd_simulation_main(int argc, char **argv, int pid);

int main(int argc, char **argv) { return cgppd_simulation_main(argc, argv, (int)getpid()); }
