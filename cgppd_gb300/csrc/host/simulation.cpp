// simulation.cpp -- see simulation.h.
#include "simulation.h"

#include <cuda_runtime.h>
#include <getopt.h>
#include <sys/stat.h>
#include <sys/types.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <fstream>
#include <tuple>
#include <sstream>

#include "../status.h"
#include "cgppd_remc.h"

namespace cgppd {

namespace {

constexpr float kBoundEnergy = -1.1844f;  // BOUND_ENERGY_VALUE, src/definitions.h:33

void mkdirs(const std::string &path)
{
    std::string cur;
    std::stringstream ss(path);
    std::string part;
    if (!path.empty() && path[0] == '/')
        cur = "/";
    while (std::getline(ss, part, '/')) {
        if (part.empty())
            continue;
        cur += part + "/";
        mkdir(cur.c_str(), 0755);
    }
}

std::vector<std::string> split_ws(const std::string &line)
{
    std::vector<std::string> out;
    std::stringstream ss(line);
    std::string w;
    while (ss >> w)
        out.push_back(w);
    return out;
}

}  // namespace

Simulation::Simulation() {}

Simulation::~Simulation()
{
    closeSamplingFiles();
    if (engine_)
        cgppd_engine_destroy(engine_);
}

void Simulation::printHelp()
{
    std::printf("Usage: cgppd -f <filename> [-h] [-p] [-q] [-v x] [-t x] [-s x] [-g x] [-z x] [-m x ] [-a x] [-e x] "
                "[-r x] [-o x] [-b x] [-n x] [-x x] [-d x]\n"
                "\t-f|--file <file>:    Input config file\n\t-q|--nosim:          Do everything except the "
                "simulation\n\t-v|--v:              Verbosity level\n\t-m|--mcsteps x   -a|--sampleafter x   "
                "-e|--resteps x   -r|--replicas x   -o|--output x   -b|--boundary x   -x|--tmax x   -n|--tmin x\n"
                "\t-t/-s/-g/-z/-d are accepted for compatibility (every replica runs on one GPU)\n");
}

// Two passes as the reference (src/Simulation.cpp:78-263): the first finds the config
// file and verbosity, the second applies command-line overrides after the file.
void Simulation::getArgs(int argc, char **argv, bool first_pass)
{
    static const struct option long_options[] = {
        {"file", required_argument, 0, 'f'},    {"help", no_argument, 0, 'h'},
        {"verbosity", required_argument, 0, 'v'}, {"preview", no_argument, 0, 'p'},
        {"nosim", no_argument, 0, 'q'},         {"threads", required_argument, 0, 't'},
        {"streams", required_argument, 0, 's'}, {"gpus", required_argument, 0, 'g'},
        {"gpuoffset", required_argument, 0, 'z'}, {"mcsteps", required_argument, 0, 'm'},
        {"sampleafter", required_argument, 0, 'a'}, {"resteps", required_argument, 0, 'e'},
        {"replicas", required_argument, 0, 'r'}, {"output", required_argument, 0, 'o'},
        {"boundary", required_argument, 0, 'b'}, {"tmax", required_argument, 0, 'x'},
        {"tmin", required_argument, 0, 'n'},    {"blockdim", required_argument, 0, 'd'},
        {0, 0, 0, 0},
    };
    const char short_options[] = "hf:pqt:s:g:z:m:a:e:r:o:b:x:n:d:v:w:";
    int opt_index = 0;
    optind = 0;  // full re-initialisation of getopt
    opterr = 0;
    if (first_pass) {
        for (;;) {
            int opt = getopt_long(argc, argv, short_options, long_options, &opt_index);
            if (opt == -1)
                break;
            if (opt == 'h') {
                printHelp();
                throw "help";
            } else if (opt == 'f') {
                parameters.file = optarg;
                parameters.inputFile = true;
            } else if (opt == 'v') {
                parameters.verbosity = std::atoi(optarg);
            }
        }
        if (!parameters.inputFile) {
            printHelp();
            throw "No configuration file provided.";
        }
        return;
    }
    char buf[512];
    for (;;) {
        int opt = getopt_long(argc, argv, short_options, long_options, &opt_index);
        if (opt == -1)
            break;
        switch (opt) {
        case 'p':
            std::fprintf(stderr, "cgppd: no OpenGL preview (headless)\n");
            break;
        case 'q': parameters.skipsimulation = true; break;
        case 't': parameters.threads = std::atoi(optarg); break;
        case 's': parameters.streams = std::atoi(optarg); break;
        case 'g': parameters.gpus = std::atoi(optarg); break;
        case 'z': parameters.gpuoffset = std::atoi(optarg); break;
        case 'm': parameters.MCsteps = std::atoi(optarg); break;
        case 'a': parameters.sampleStartsAfter = std::atoi(optarg); break;
        case 'e': parameters.REsteps = std::atoi(optarg); break;
        case 'r': parameters.replicas = std::atoi(optarg); break;
        case 'o':
            std::snprintf(buf, sizeof(buf), "%s_%d", optarg, parameters.pid);
            parameters.prefix = buf;
            break;
        case 'b': parameters.bound = (float)std::atof(optarg); break;
        case 'x': parameters.temperatureMax = (float)std::atof(optarg); break;
        case 'n': parameters.temperatureMin = (float)std::atof(optarg); break;
        case 'd':
            parameters.cuda_blockSize = std::atoi(optarg);
            parameters.auto_blockdim = false;
            break;
        default: break;
        }
    }
}

// Sections: parameters (`key value`), `files`, `crowders`, `segments`
// (src/Simulation.cpp:265-453).
void Simulation::loadArgsFromFile()
{
    std::ifstream in(parameters.file.c_str());
    if (!in.good())
        throw "Failed to open config file.";
    enum { kParams, kMolecules, kCrowders, kSegments } section = kParams;
    std::string line;
    char buf[512];
    while (std::getline(in, line)) {
        if (!line.empty() && line.back() == '\r')
            line.pop_back();
        if (line.empty() || line[0] == '#')
            continue;
        if (line == "files") {
            section = kMolecules;
        } else if (line == "crowders") {
            section = kCrowders;
        } else if (line == "segments") {
            section = kSegments;
        } else if (section == kMolecules || section == kCrowders) {
            MolData m;
            char flag = 0, pdb[256] = {0}, name[256] = {0};
            int got = std::sscanf(line.c_str(), "%c(%f,%f,%f) r(%f,%f,%f,%f) %255s %255s", &flag, &m.px, &m.py, &m.pz,
                                  &m.rx, &m.ry, &m.rz, &m.ra, pdb, name);
            m.translate = (flag == 't');
            if (got < 8) {
                std::fprintf(stderr, "cgppd: unable to parse molecule: %s\n", line.c_str());
                continue;
            }
            m.pdbfilename = pdb;
            m.name = name;
            m.crowder = (section == kCrowders);
            if (section == kMolecules)
                parameters.nonCrowders++;
            parameters.mdata.push_back(m);
            if (!m.name.empty())
                parameters.mdata_map[m.name] = (int)parameters.mdata.size() - 1;
        } else if (section == kSegments) {
            std::vector<std::string> w = split_ws(line);
            if (w.size() < 2)
                continue;
            auto it = parameters.mdata_map.find(w[0]);
            if (it == parameters.mdata_map.end())
                throw "Segment refers to an unknown molecule name.";
            MolData &md = parameters.mdata[it->second];
            if (w[1] == "all") {
                md.all_flexible = true;
            } else {
                std::vector<int> seg;
                for (size_t k = 1; k < w.size(); ++k)
                    seg.push_back(std::atoi(w[k].c_str()) - 1);
                md.segments.push_back(seg);
            }
        } else {
            std::vector<std::string> w = split_ws(line);
            if (w.empty())
                continue;
            const std::string &key = w[0];
            const char *v = w.size() > 1 ? w[1].c_str() : "0";
            if (key == "gpus") parameters.gpus = std::atoi(v);
            else if (key == "gpuoffset") parameters.gpuoffset = std::atoi(v);
            else if (key == "streams") parameters.streams = std::atoi(v);
            else if (key == "threads") parameters.threads = std::atoi(v);
            else if (key == "mcsteps") parameters.MCsteps = std::atoi(v);
            else if (key == "resteps") parameters.REsteps = std::atoi(v);
            else if (key == "temperaturemax") parameters.temperatureMax = (float)std::atof(v);
            else if (key == "temperaturemin") parameters.temperatureMin = (float)std::atof(v);
            else if (key == "boundary") parameters.bound = (float)std::atof(v);
            else if (key == "replicas") parameters.replicas = std::atoi(v);
            else if (key == "samplefrequency") parameters.sampleFrequency = std::atoi(v);
            else if (key == "sampleafter") parameters.sampleStartsAfter = std::atoi(v);
            else if (key == "prefix") {
                std::snprintf(buf, sizeof(buf), "%s_%d", v, parameters.pid);
                parameters.prefix = buf;
            } else if (key == "title") {
                std::string t;
                for (size_t k = 1; k < w.size(); ++k)
                    t += (k > 1 ? " " : "") + w[k];
                parameters.title = t;
            } else if (key == "translatemin") parameters.translateMin = (float)std::atof(v);
            else if (key == "translatemax") parameters.translateMax = (float)std::atof(v);
            else if (key == "rotatemin") parameters.rotateMin = (float)std::atof(v);
            else if (key == "rotatemax") parameters.rotateMax = (float)std::atof(v);
            else if (key == "moveweights" && w.size() >= 5) {
                for (int k = 0; k < 4; ++k)
                    parameters.moveWeights[k] = (float)std::atof(w[1 + k].c_str());
            } else if (key == "seed") parameters.seed = std::strtoull(v, nullptr, 10);
            else if (key == "datadir") parameters.dataDir = v;
            else if (key == "repulsivecrowding") parameters.repulsiveCrowding = std::atoi(v) != 0;
            else std::fprintf(stderr, "cgppd: unknown parameter: %s\n", key.c_str());
        }
    }
}

// src/Simulation.cpp:455-514
void Simulation::check_and_modify_parameters()
{
    if (parameters.bound <= 0)
        parameters.bound = 150.0f;
    if (parameters.temperatureMax < parameters.temperatureMin) {
        float tmp = parameters.temperatureMax;
        parameters.temperatureMax = parameters.temperatureMin;
        parameters.temperatureMin = tmp;
    }
    if (parameters.threads > parameters.replicas)
        parameters.threads = parameters.replicas;
    if (parameters.threads < 1)
        parameters.threads = 1;
    parameters.max_replicas_per_thread =
        (int)std::ceil((float)parameters.replicas / (float)parameters.threads);
    const int spaces = parameters.max_replicas_per_thread * parameters.threads - parameters.replicas;
    if (spaces / parameters.max_replicas_per_thread)
        throw "Wasted threads.";
    int available = 0;
    cudaGetDeviceCount(&available);
    if (parameters.gpuoffset >= available)
        throw "GPU allocation impossible.";
    if (parameters.gpus + parameters.gpuoffset > available)
        parameters.gpus = available - parameters.gpuoffset;
    if (parameters.REsteps < 1 || parameters.MCsteps < parameters.REsteps)
        throw "mcsteps must be at least resteps (one MC step per exchange block).";
}

void Simulation::load_torsions(const std::string &path)
{
    torsionV.assign(20 * 20 * 4, 0.0);
    torsionPhase.assign(20 * 20 * 4, 0.0);
    std::ifstream in(path.c_str());
    if (!in.good())
        throw "Failed to open torsional data file.";
    std::string line;
    while (std::getline(in, line)) {
        if (line.empty() || line[0] == '#')
            continue;
        char a0[8] = {0}, a1[8] = {0};
        double v = 0, sigma = 0;
        int n = 0;
        if (std::sscanf(line.c_str(), "%3s %3s %lf %d %lf", a0, a1, &v, &n, &sigma) != 5 || n < 1 || n > 4)
            continue;
        const int i = aminoAcidData.getAminoAcidIndex(a0), j = aminoAcidData.getAminoAcidIndex(a1);
        if (i < 0 || j < 0)
            throw "Unknown residue name in torsional data file.";
        torsionV[(i * 20 + j) * 4 + n - 1] = v;
        torsionPhase[(i * 20 + j) * 4 + n - 1] = sigma / 57.29577951308232;  // degrees to radians
    }
}

void Simulation::init(int argc, char **argv, int pid)
{
    parameters.pid = pid;
    getArgs(argc, argv, true);
    loadArgsFromFile();
    getArgs(argc, argv, false);
    outdir = "output/" + parameters.prefix;
    mkdirs(outdir + "/pdb");
    initSamplingFiles();
    check_and_modify_parameters();

    const std::string dd = parameters.dataDir;
    aminoAcidData.init((dd + "/AminoAcids").c_str(), (dd + "/pair_potentials_MJ1996").c_str());
    bool flexible = false;
    for (auto &m : parameters.mdata)
        flexible = flexible || m.all_flexible || !m.segments.empty();
    if (flexible)
        load_torsions(dd + "/torsional_pair_potentials");

    molecules.clear();
    for (auto &m : parameters.mdata) {
        int chains = 1;
        std::vector<PdbResidue> res = read_pdb(m.pdbfilename, aminoAcidData, &chains);
        molecules.push_back(place_molecule(res, chains, m.translate, m.px, m.py, m.pz, m.rx, m.ry, m.rz, m.ra,
                                           parameters.bound));
    }
    if (molecules.empty())
        throw "No molecules loaded.";

    // ladders (src/Simulation.cpp:590-598, src/Replica.cpp:79-98)
    const int R = parameters.replicas;
    const double den = R > 1 ? 1.0 / (double)(R - 1) : 0.0;
    geometricTemperature = std::pow((double)(parameters.temperatureMax / parameters.temperatureMin), den);
    geometricTranslate = std::pow((double)(parameters.translateMax / parameters.translateMin), den);
    geometricRotation = std::pow((double)(parameters.rotateMax / parameters.rotateMin), den);
    std::vector<float> temps(R), tsteps(R);
    std::vector<double> rsteps(R);
    for (int i = 0; i < R; ++i) {
        temps[i] = (float)(parameters.temperatureMin * std::pow(geometricTemperature, i));
        rsteps[i] = parameters.rotateMin * std::pow(geometricRotation, i);
        tsteps[i] = (float)(parameters.translateMin * std::pow(geometricTranslate, i));
        position_of_temperature[temps[i]] = i;
        temperature[i] = temps[i];
    }

    unsigned long long seed = parameters.seed;
    if (seed == 0)
        seed = (unsigned long long)std::chrono::high_resolution_clock::now().time_since_epoch().count();
    engine_ = cgppd_engine_create(&aminoAcidData.LJpotentials[0][0], 20, flexible ? torsionV.data() : nullptr,
                                  flexible ? torsionPhase.data() : nullptr, 20, seed);
    if (!engine_)
        throw "Engine creation failed.";
    cgppd_sim_params p{};
    p.n_replicas = R;
    p.box = parameters.bound;
    p.temperatures = temps.data();
    p.translate_steps = tsteps.data();
    p.rotate_steps = rsteps.data();
    for (int k = 0; k < 4; ++k)
        p.move_weights[k] = parameters.moveWeights[k];
    p.rigid_rotate_prob = 0.5f;  // translate_rotate_bernoulli_bias, src/definitions.h:34
    p.sample_frequency = parameters.sampleFrequency;
    p.sample_after = parameters.sampleStartsAfter;
    p.bound_threshold = kBoundEnergy;
    p.repulsive_crowding = parameters.repulsiveCrowding ? 1 : 0;
    if (cgppd_engine_add_simulation(engine_, &p) < 0)
        throw "Engine set-up failed.";
    for (size_t k = 0; k < molecules.size(); ++k) {
        const PlacedMolecule &pm = molecules[k];
        const MolData &md = parameters.mdata[k];
        const int n = (int)pm.residues.size();
        std::vector<int> types(n), seq(n), cidx(n);
        std::vector<float> q(n), s(n);
        std::vector<char> chains(n);
        for (int i = 0; i < n; ++i) {
            const PdbResidue &r = pm.residues[i];
            types[i] = r.type;
            q[i] = aminoAcidData.data[r.type].electrostaticCharge;  // per type, src/Molecule.cpp:553-555
            s[i] = aminoAcidData.data[r.type].vanderWaalRadius;
            seq[i] = r.res_seq;
            cidx[i] = r.chain_index;
            chains[i] = r.chain;
        }
        std::vector<int> seglen, segres;
        for (auto &sg : md.segments) {
            seglen.push_back((int)sg.size());
            segres.insert(segres.end(), sg.begin(), sg.end());
        }
        if (cgppd_engine_add_molecule(engine_, 0, n, pm.pos.data(), types.data(), q.data(), s.data(), chains.data(),
                                      seq.data(), cidx.data(), pm.num_chains, md.all_flexible ? 1 : 0,
                                      md.crowder ? 1 : 0, (int)md.segments.size(), seglen.data(), segres.data(),
                                      pm.center) < 0)
            throw "Molecule set-up failed (check segment indices).";
    }
    if (cgppd_engine_finalize(engine_, 0, 0) != 0)
        throw "Engine finalize failed.";
}

void Simulation::initSamplingFiles()
{
    auto open = [&](const char *name, FILE **f) {
        const std::string path = outdir + "/" + name;
        *f = std::fopen(path.c_str(), "a+");
        if (!*f)
            *f = std::fopen(path.c_str(), "wt");
        if (!*f)
            throw "Could not open / create sampling file.";
    };
    open("fractionBound", &fractionBoundFile);
    open("boundconformations", &boundConformationsFile);
    open("acceptance_ratios", &acceptanceRatioFile);
    open("exchange_freq", &exchangeFrequencyFile);
}

void Simulation::closeSamplingFiles()
{
    for (FILE **f : {&fractionBoundFile, &boundConformationsFile, &acceptanceRatioFile, &exchangeFrequencyFile})
        if (*f) {
            std::fclose(*f);
            *f = nullptr;
        }
}

void Simulation::writeFileIndex()
{
    FILE *f = std::fopen((outdir + "/fileindex").c_str(), "w");
    if (!f)
        throw "Could not write the file index.";
    std::fprintf(f, "index molecule_file_path crowder(Y/N)\n");
    for (size_t i = 0; i < parameters.mdata.size(); ++i)
        std::fprintf(f, "%2d %s %s", (int)i, parameters.mdata[i].pdbfilename.c_str(),
                     parameters.mdata[i].crowder ? "Y\n" : "N\n");
    std::fclose(f);
}

void Simulation::writeSamplingFileHeaders()
{
    std::fprintf(fractionBoundFile, "# Fraction Bound\n#Iteration InstantaneousAve CumulativeAve\n");
    std::fprintf(boundConformationsFile, "# iteration; complex free energy (replica free energy); temperature;\n# "
                                         "molecule: pdb file; 1 line per other molecule in the bound state\n");
    std::fprintf(acceptanceRatioFile, "# Iteration AcceptanceRatio\n");
    std::fprintf(exchangeFrequencyFile, "# Iteration continous_ratio, inst_ratio\n");
    std::fprintf(fractionBoundFile, "Iteration:  ");
    std::fprintf(acceptanceRatioFile, "Iteration:  ");
    for (auto &kv : position_of_temperature) {
        std::fprintf(fractionBoundFile, "%0.1fKi %0.1fKc ", kv.first, kv.first);
        std::fprintf(acceptanceRatioFile, "%0.1fKi %0.1fKc ", kv.first, kv.first);
    }
    std::fprintf(fractionBoundFile, " \n");
    std::fprintf(acceptanceRatioFile, "\n");
}

// One line of fractionBound and acceptance_ratios from device report row `row`.
void Simulation::write_report_row(int label, int row)
{
    const int R = parameters.replicas;
    std::vector<float> rep(4 * R);
    cgppd_engine_get_report(engine_, 0, row, rep.data(), nullptr);
    std::fprintf(fractionBoundFile, "%9d: ", label);
    std::fprintf(acceptanceRatioFile, "%9d: ", label);
    for (int t = 0; t < R; ++t) {  // temperature-ladder order (src/Simulation.cpp:757-762)
        std::fprintf(fractionBoundFile, "| %6.4f %6.4f ", rep[4 * t], rep[4 * t + 1]);
        std::fprintf(acceptanceRatioFile, "| %6.4f %6.4f ", rep[4 * t + 2], rep[4 * t + 3]);
    }
    std::fprintf(fractionBoundFile, "\n");
    std::fprintf(acceptanceRatioFile, "\n");
    std::fflush(fractionBoundFile);
    std::fflush(acceptanceRatioFile);
}

// Simulation::exchange_frequency (src/Simulation.cpp:876-888).
void Simulation::exchange_frequency(int steps, int row)
{
    int ex[2] = {0, 0};
    cgppd_engine_get_report(engine_, 0, row, nullptr, ex);
    totalExchanges += ex[0];
    totalTests += ex[1];
    const float frac = (float)ex[0] / (float)ex[1];
    const float acc = (float)totalExchanges / (float)totalTests;
    std::fprintf(exchangeFrequencyFile, "%10d %6.4f %6.4f\n", steps, acc, frac);
}

// The lines Replica::sample writes to boundconformations (src/Replica.cpp:1083-1091),
// from the device's sample log: "step; E_nc (E); T" and the name of the sample's PDB
// file, in the order one reference thread writes them (block, replica slot, step).  The
// PDB files themselves are not written.
void Simulation::write_samples(int steps_per_block, int cap)
{
    int R = 0;
    cgppd_engine_sim_info(engine_, 0, nullptr, nullptr, &R);
    std::vector<int> counts(R), step((size_t)R * cap);
    std::vector<double> enc((size_t)R * cap), pot((size_t)R * cap);
    std::vector<float> temp((size_t)R * cap);
    if (cgppd_engine_take_samples(engine_, 0, counts.data(), enc.data(), pot.data(), temp.data(), step.data()) != 0)
        throw "MC run failed.";
    std::vector<std::tuple<int, int, int, size_t>> order;
    for (int r = 0; r < R; ++r)
        for (int k = 0; k < counts[r]; ++k) {
            const size_t o = (size_t)r * cap + k;
            order.emplace_back(step[o] / steps_per_block, r, step[o], o);
        }
    std::sort(order.begin(), order.end());
    // every sample's conformation (the reference's build records all samples,
    // src/definitions.h:36): the non-crowder molecules, which lead the replica
    const int nres = sample_residues();
    std::vector<float> xyz((size_t)R * cap * nres * 3);
    if (nres > 0 && cgppd_engine_take_sample_xyz(engine_, 0, xyz.data()) != 0)
        throw "MC run failed.";
    // the residues' records: types, numbers, replica-wide chains (src/Geometry.cpp:256-297),
    // molecules
    std::vector<int> types, seq, chain, mol;
    for (size_t k = 0, chain_base = 0; k < molecules.size() && !parameters.mdata[k].crowder; ++k) {
        for (const auto &r : molecules[k].residues) {
            types.push_back(r.type);
            seq.push_back(r.res_seq);
            chain.push_back((int)chain_base + r.chain_index);
            mol.push_back((int)k);
        }
        chain_base += molecules[k].num_chains;
    }
    char name[512];
    for (const auto &x : order) {
        const size_t o = std::get<3>(x);
        std::snprintf(name, sizeof(name), "%s/pdb/sample_%d_%0.1fK_%5.2f.pdb", outdir.c_str(), step[o],
                      (double)temp[o], enc[o]);
        std::fprintf(boundConformationsFile, "%d; %0.5f (%0.5f); %0.1f\n%s\n", step[o], enc[o], pot[o],
                     (double)temp[o], name);
        if (nres > 0) {
            FILE *f = std::fopen(name, "w");
            if (f) {
                write_sample_pdb(f, parameters.prefix.c_str(), temp[o], step[o], pot[o], nres, xyz.data() + o * nres * 3,
                                 types.data(), seq.data(), chain.data(), mol.data(), aminoAcidData);
                std::fclose(f);
            }
        }
    }
    std::fflush(boundConformationsFile);
}

// Residues of the molecules before the first crowder (the part of a replica a sample
// PDB holds).
int Simulation::sample_residues() const
{
    int n = 0;
    for (size_t k = 0; k < molecules.size() && !parameters.mdata[k].crowder; ++k)
        n += (int)molecules[k].residues.size();
    return n;
}

// Simulation::run (src/Simulation.cpp:709-873): REsteps blocks of MCsteps/REsteps MC
// steps with REsteps-1 exchanges in between, all on the device; the per-exchange
// reports are read back afterwards and written in the reference's formats.
void Simulation::run()
{
    writeFileIndex();
    writeSamplingFileHeaders();
    if (parameters.skipsimulation)
        return;
    const int K = parameters.MCsteps / parameters.REsteps;
    const int RE = parameters.REsteps;
    // the samples' lines of boundconformations come from the device's sample log, read
    // back after chunks of blocks small enough for the log
    const int freq = parameters.sampleFrequency;
    const int per_block = freq > 0 ? (K + freq - 1) / freq : 0;
    int chunk = RE;
    if (per_block > 0) {
        // records per replica held between reads: at most 4096, and the samples'
        // coordinates within 256 MB, but always one block's
        const long long per_record = (long long)parameters.replicas * sample_residues() * 16;
        const long long fit = per_record > 0 ? (256LL << 20) / per_record : 4096;
        const int records = std::max(per_block, (int)std::min<long long>(4096, fit));
        chunk = std::max(1, std::min(RE, records / per_block));
        if (cgppd_engine_set_sample_snapshots(engine_, sample_residues()) != 0 ||
            cgppd_engine_set_sample_log(engine_, chunk * per_block) != 0)
            throw "MC run failed.";
    }
    for (int b = 0; b < RE; b += chunk) {
        const int nb = std::min(chunk, RE - b);
        if (cgppd_engine_run(engine_, nb, K, (b + nb < RE) ? 1 : 0, nullptr) != 0)
            throw "MC run failed.";
        if (per_block > 0)
            write_samples(K, chunk * per_block);
    }
    if (cgppd_engine_final_report(engine_, RE - 1, nullptr) != 0 || cgppd_engine_synchronize(engine_) != 0)
        throw "MC run failed.";
    for (int steps = 1; steps < RE; ++steps) {
        if ((long long)K * (steps - 1) >= parameters.sampleStartsAfter)
            write_report_row(K * steps, steps - 1);
        exchange_frequency(steps, steps - 1);
    }
    write_report_row(parameters.MCsteps, RE - 1);
    // final coordinates of the lowest-temperature replica in the reference PDB format
    const int R = parameters.replicas;
    std::vector<int> tindex(R);
    cgppd_engine_get_replicas(engine_, 0, nullptr, nullptr, nullptr, tindex.data(), nullptr);
    int slot = 0;
    for (int r = 0; r < R; ++r)
        if (tindex[r] == 0)
            slot = r;
    int N = 0;
    cgppd_engine_sim_info(engine_, 0, &N, nullptr, nullptr);
    std::vector<float> xyz(3 * N);
    cgppd_engine_get_state(engine_, 0, slot, xyz.data(), nullptr, nullptr);
    FILE *f = std::fopen((outdir + "/pdb/final_lowest_temperature.pdb").c_str(), "w");
    if (f) {
        std::fprintf(f, "REMARK simulation: %s \n", parameters.prefix.c_str());
        std::fprintf(f, "REMARK temperature: %5.1f \n", temperature[0]);
        int counter = 0, off = 0, chain_base = 0;
        for (size_t k = 0; k < molecules.size(); ++k) {
            if (!parameters.mdata[k].crowder)
                write_pdb_atoms(f, molecules[k].residues, xyz.data() + 3 * off, aminoAcidData, &counter, chain_base);
            chain_base += molecules[k].num_chains;
            off += (int)molecules[k].residues.size();
        }
        std::fprintf(f, "END \n");
        std::fclose(f);
    }
    closeSamplingFiles();
}

}  // namespace cgppd

// ------------------------------------------------------------------ C entry points

// Parse only (no GPU): mode bit 0 runs the first command-line pass, bit 1 reads the
// config file, bit 2 runs the second command-line pass.  The resulting parameters are
// written to buf as `key=value` lines.  Returns 0, or 1 with the message in buf.
extern "C" int cgppd_args_dump(int argc, char **argv, int mode, char *buf, int buflen)
{
    cgppd::Simulation s;
    std::ostringstream o;
    try {
        if ((mode & 8) && argc > 1) {  // config file given directly as argv[1]
            s.parameters.file = argv[1];
            s.parameters.inputFile = true;
        }
        if (mode & 1)
            s.getArgs(argc, argv, true);
        if (mode & 2)
            s.loadArgsFromFile();
        if (mode & 4)
            s.getArgs(argc, argv, false);
    } catch (const char *msg) {
        std::snprintf(buf, (size_t)buflen, "%s", msg);
        return 1;
    }
    const cgppd::ArgData &p = s.parameters;
    o << "viewConditions=" << p.viewConditions << "\nskipsimulation=" << p.skipsimulation
      << "\ncuda_blockSize=" << p.cuda_blockSize << "\nauto_blockdim=" << p.auto_blockdim << "\nthreads=" << p.threads
      << "\nstreams=" << p.streams << "\ngpus=" << p.gpus << "\ngpuoffset=" << p.gpuoffset << "\nMCsteps=" << p.MCsteps
      << "\nREsteps=" << p.REsteps << "\nreplicas=" << p.replicas << "\nsampleFrequency=" << p.sampleFrequency
      << "\nsampleStartsAfter=" << p.sampleStartsAfter << "\ninputFile=" << p.inputFile
      << "\nnonCrowders=" << p.nonCrowders << "\npid=" << p.pid << "\nresume=" << p.resume << "\nbound=" << p.bound
      << "\ntemperatureMin=" << p.temperatureMin << "\ntemperatureMax=" << p.temperatureMax << "\nprefix=" << p.prefix
      << "\nfile=" << p.file << "\ntitle=" << p.title << "\nmolecules=" << p.mdata.size()
      << "\nnamed=" << p.mdata_map.size() << "\nrepulsiveCrowding=" << p.repulsiveCrowding << "\n";
    for (size_t i = 0; i < p.mdata.size(); ++i) {
        const cgppd::MolData &m = p.mdata[i];
        o << "mol" << i << "=" << m.pdbfilename << " " << (m.name.empty() ? "-" : m.name) << " " << m.translate << " "
          << m.px << " " << m.py << " " << m.pz << " " << m.rx << " " << m.ry << " " << m.rz << " " << m.ra << " "
          << m.crowder << " " << m.all_flexible << " " << m.segments.size();
        for (auto &sg : m.segments) {
            o << " [";
            for (size_t k = 0; k < sg.size(); ++k)
                o << (k ? "," : "") << sg[k];
            o << "]";
        }
        o << "\n";
    }
    std::snprintf(buf, (size_t)buflen, "%s", o.str().c_str());
    return 0;
}

// main() of the reference (src/main.cpp:3-44) as a library call: init + run, with the
// reference's "Aborting" on a thrown message.  Returns 0 on success, 1 on failure.
extern "C" int cgppd_simulation_main(int argc, char **argv, int pid)
{
    try {
        cgppd::Simulation s;
        s.init(argc, argv, pid);
        s.run();
    } catch (const char *msg) {
        std::fprintf(stderr, "cgppd: %s\nAborting.\n", msg);
        return 1;
    }
    return 0;
}
