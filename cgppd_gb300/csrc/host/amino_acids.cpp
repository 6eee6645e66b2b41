// amino_acids.cpp -- loaders for the residue-type file and the contact table.
#include "amino_acids.h"
#include "cgppd_amino_acids.h"

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

AminoAcid::AminoAcid() : shortSymbol(0), vanderWaalRadius(0.0f), electrostaticCharge(0.0f), index(0)
{
    std::memset(name, 0, sizeof(name));
    std::memset(sname, 0, sizeof(sname));
}

AminoAcid::~AminoAcid() {}

AminoAcids::AminoAcids() : clean(false)
{
    std::memset(LJpotentials, 0, sizeof(LJpotentials));
}

AminoAcids::~AminoAcids() {}

void AminoAcids::init(const char *aminoAcidFile, const char *ljFile)
{
    clean = loadAminoAcidData(aminoAcidFile) && loadLJPotentialData(ljFile);
}

// Records are five lines each (name, short name, one-letter symbol, vdW radius,
// charge); blank lines and '#' comments separate them.  Records fill data[] in file
// order, which defines the residue-type index.
bool AminoAcids::loadAminoAcidData(const char *path)
{
    std::ifstream in(path);
    if (!in.good())
        throw "Failed to open amino acid data file.";
    std::vector<std::string> lines;
    std::string ln;
    while (std::getline(in, ln))
        lines.push_back(ln);
    int i = 0;
    for (size_t k = 0; k < lines.size() && i < 20;) {
        const std::string &l = lines[k];
        if (l.empty() || l[0] == '#') {
            ++k;
            continue;
        }
        if (k + 4 >= lines.size())
            break;
        std::memset(data[i].name, 0, 20);
        std::memset(data[i].sname, 0, 4);
        std::strncpy(data[i].name, l.c_str(), std::min<size_t>(l.size(), 19));
        const std::string &s = lines[k + 1];
        std::strncpy(data[i].sname, s.c_str(), std::min<size_t>(s.size(), 3));
        data[i].shortSymbol = lines[k + 2].empty() ? 0 : lines[k + 2][0];
        data[i].vanderWaalRadius = (float)std::atof(lines[k + 3].c_str());
        float q = 0.0f;
        std::sscanf(lines[k + 4].c_str(), "%f", &q);
        data[i].electrostaticCharge = q;
        data[i].index = i;
        ++i;
        k += 5;
    }
    return i == 20;
}

// Upper-triangular table: one label row, then row k holds columns k..19.  Labels are
// mapped to type indices, and the table is stored symmetric.
bool AminoAcids::loadLJPotentialData(const char *path)
{
    std::ifstream in(path);
    if (!in.good())
        throw "Failed to open LJ potential data file";
    int labels[20];
    int nlabels = 0;
    int start = 0;
    std::string ln;
    while (std::getline(in, ln)) {
        if (ln.empty() || ln[0] == '#')
            continue;
        std::vector<std::string> tok;
        size_t p = 0;
        while (p < ln.size()) {
            while (p < ln.size() && std::isspace((unsigned char)ln[p]))
                ++p;
            size_t q = p;
            while (q < ln.size() && !std::isspace((unsigned char)ln[q]))
                ++q;
            if (q > p)
                tok.push_back(ln.substr(p, q - p));
            p = q;
        }
        if (tok.empty())
            continue;
        if (nlabels == 0) {
            for (size_t t = 0; t < tok.size() && nlabels < 20; ++t)
                labels[nlabels++] = getAminoAcidIndex(tok[t].c_str());
            continue;
        }
        if (start >= 20)
            break;
        for (int j = start; j < 20 && (size_t)(j - start + 1) < tok.size(); ++j) {
            float e = 0.0f;
            std::sscanf(tok[j - start + 1].c_str(), "%f", &e);
            int a = labels[start], b = labels[j];
            if (a < 0 || b < 0)
                throw "Unknown residue label in LJ potential data file";
            LJpotentials[a][b] = e;
            LJpotentials[b][a] = e;
        }
        ++start;
    }
    return start == 20;
}

int AminoAcids::getAminoAcidIndex(const char *nm) const
{
    size_t len = std::strlen(nm);
    if (len < 1)
        return -1;
    char key[24] = {0};
    if (len == 3) {
        key[0] = (char)std::toupper(nm[0]);
        key[1] = (char)std::tolower(nm[1]);
        key[2] = (char)std::tolower(nm[2]);
        for (int i = 19; i >= 0; --i)
            if (std::strcmp(key, data[i].sname) == 0)
                return i;
    } else if (len == 1) {
        char c = (char)std::toupper(nm[0]);
        for (int i = 19; i >= 0; --i)
            if (c == data[i].shortSymbol)
                return i;
    } else {
        std::strncpy(key, nm, 23);
        key[0] = (char)std::toupper(key[0]);
        for (int i = 19; i >= 0; --i)
            if (std::strcmp(key, data[i].name) == 0)
                return i;
    }
    return -1;
}

// ------------------------------------------------------------------ C helpers
extern "C" {

AminoAcids *cgppd_aminoacids_create(void) { return new AminoAcids(); }

void cgppd_aminoacids_destroy(AminoAcids *a) { delete a; }

int cgppd_aminoacids_load(AminoAcids *a, const char *aa_path, const char *lj_path)
{
    try {
        a->init(aa_path, lj_path);
    } catch (const char *msg) {
        std::fprintf(stderr, "cgppd: %s\n", msg);
        return -1;
    }
    return a->clean ? 0 : -1;
}

void cgppd_aminoacids_set(AminoAcids *a, int i, const char *name, const char *sname, char symbol,
                          float radius, float charge)
{
    std::memset(a->data[i].name, 0, 20);
    std::memset(a->data[i].sname, 0, 4);
    std::strncpy(a->data[i].name, name, 19);
    std::strncpy(a->data[i].sname, sname, 3);
    a->data[i].shortSymbol = symbol;
    a->data[i].vanderWaalRadius = radius;
    a->data[i].electrostaticCharge = charge;
    a->data[i].index = i;
}

void cgppd_aminoacids_set_table(AminoAcids *a, const float *table400)
{
    std::memcpy(&a->LJpotentials[0][0], table400, sizeof(float) * 400);
    a->clean = true;
}

void cgppd_aminoacids_get_table(const AminoAcids *a, float *table400)
{
    std::memcpy(table400, &a->LJpotentials[0][0], sizeof(float) * 400);
}

int cgppd_aminoacids_index(const AminoAcids *a, const char *name) { return a->getAminoAcidIndex(name); }

size_t cgppd_aminoacids_lj_offset(void)
{
    static AminoAcids probe;
    return (size_t)(reinterpret_cast<const char *>(&probe.LJpotentials[0][0]) - reinterpret_cast<const char *>(&probe));
}

size_t cgppd_aminoacids_sizeof(void) { return sizeof(AminoAcids); }
}
