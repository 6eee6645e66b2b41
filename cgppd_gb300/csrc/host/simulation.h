// simulation.h -- the REMC driver with the reference's configuration grammar and
// output files, running every replica on the GPU engine.
//
// Same argfile format (src/Simulation.cpp:265-453), command-line options
// (src/Simulation.cpp:78-263), parameter checks (:455-514), temperature and step
// ladders (:590-598, src/Replica.cpp:79-98) and output files (fileindex, fractionBound,
// acceptance_ratios, exchange_freq, boundconformations: src/Simulation.cpp:536-548,
// :743-768, :876-888, :1114-1194) as the reference's Simulation.
#pragma once

#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "amino_acids.h"
#include "pdb.h"

struct cgppd_engine;

namespace cgppd {

struct MolData {
    std::string pdbfilename, name;
    float px = 0, py = 0, pz = 0;
    bool translate = false;
    float rx = 0, ry = 0, rz = 0, ra = 0;
    bool crowder = false, all_flexible = false;
    std::vector<std::vector<int>> segments;  // 0-based residue indices
};

// argdata (src/structures.h:78-127) with the reference defaults (src/definitions.h).
struct ArgData {
    bool viewConditions = false, skipsimulation = false;
    int cuda_blockSize = 64;
    bool auto_blockdim = true;
    int threads = 1, streams = 1, gpus = 1, gpuoffset = 0;
    int max_replicas_per_thread = 0;
    int MCsteps = 5000, REsteps = 10, replicas = 20;
    float bound = 150.0f;
    int sampleFrequency = 5000, sampleStartsAfter = 5000, checkpointFrequency = 10000;
    std::string prefix, title, file;
    bool inputFile = false;
    int nonCrowders = 0;
    float temperatureMin = 250.0f, temperatureMax = 500.0f;
    int pid = 0;
    bool resume = false;
    int verbosity = 1;
    std::vector<MolData> mdata;
    std::map<std::string, int> mdata_map;
    // Extensions (absent keys keep the reference's compiled-in values): translate and
    // rotate step ladders (src/definitions.h:28-32), move weights of flexible molecules
    // (src/definitions.h:86-89), random seed, data directory.
    float translateMin = 0.5f, translateMax = 2.0f;
    float rotateMin = 0.2f, rotateMax = 0.4f;
    float moveWeights[4] = {1.0f, 1.0f, 1.0f, 1.0f};
    unsigned long long seed = 0;  // 0: from the clock, as the reference seeds its RNGs
    std::string dataDir = "data";
    bool repulsiveCrowding = false;  // REPULSIVE_CROWDING (src/definitions.h:18), off there
};

class Simulation {
public:
    ArgData parameters;
    AminoAcids aminoAcidData;
    std::vector<double> torsionV, torsionPhase;  // [20][20][4]
    std::vector<PlacedMolecule> molecules;
    std::map<float, int> position_of_temperature;
    std::map<int, float> temperature;
    double geometricTemperature = 1, geometricTranslate = 1, geometricRotation = 1;
    std::string outdir;

    Simulation();
    ~Simulation();

    void getArgs(int argc, char **argv, bool first_pass);
    void loadArgsFromFile();
    void check_and_modify_parameters();
    void init(int argc, char **argv, int pid);
    void run();
    void printHelp();

    cgppd_engine *engine() { return engine_; }

private:
    void load_torsions(const std::string &path);
    void writeFileIndex();
    void initSamplingFiles();
    void writeSamplingFileHeaders();
    void closeSamplingFiles();
    void write_report_row(int mcsteps_label, int row);
    void exchange_frequency(int steps, int row);
    void write_samples(int steps_per_block, int log_capacity);
    int sample_residues() const;

    cgppd_engine *engine_ = nullptr;
    FILE *fractionBoundFile = nullptr, *boundConformationsFile = nullptr, *acceptanceRatioFile = nullptr,
         *exchangeFrequencyFile = nullptr;
    long long totalExchanges = 0, totalTests = 0;
};

}  // namespace cgppd
