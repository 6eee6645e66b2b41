/*
 * cgppd_simulation.h -- the REMC program as a library call.
 *
 * The reference's executable (src/main.cpp:3-44) builds a Simulation from the command
 * line and the argfile and runs it on host threads.  Here the same command line and
 * argfile drive the GPU engine; output files are written in the reference's formats
 * under output/<prefix>/.  The `cgppd` executable built next to the library is
 * `main(argc, argv) { return cgppd_simulation_main(argc, argv, getpid()); }`.
 */
#ifndef CGPPD_SIMULATION_H_
#define CGPPD_SIMULATION_H_

#ifdef __cplusplus
extern "C" {
#endif

/* Replaces main + Simulation::init + Simulation::run (src/main.cpp:3-44,
 * src/Simulation.cpp:516-873).  Returns 0 on success, 1 after printing the thrown
 * message and "Aborting." as the reference does. */
int cgppd_simulation_main(int argc, char **argv, int pid);

/* Parse only, no GPU (Simulation::getArgs / loadArgsFromFile, src/Simulation.cpp:78-453):
 * mode bit 0 = first command-line pass, bit 1 = read the config file, bit 2 = second
 * command-line pass, bit 3 = take argv[1] as the config file path.  The parameters are
 * written to buf as `key=value` lines; returns 0, or 1 with the error message in buf. */
int cgppd_args_dump(int argc, char **argv, int mode, char *buf, int buflen);

#ifdef __cplusplus
}
#endif

#endif /* CGPPD_SIMULATION_H_ */
