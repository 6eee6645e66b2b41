// pdb.cpp -- see pdb.h.
#include "pdb.h"

#include "../status.h"
#include "cgppd_pdb.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>

namespace cgppd {

std::vector<PdbResidue> read_pdb(const std::string &path, const AminoAcids &aa, int *num_chains)
{
    std::ifstream in(path.c_str());
    if (!in.good())
        throw "Failed to open PDB file.";
    std::vector<PdbResidue> out;
    int chains = 0;
    std::string ln;
    while (std::getline(in, ln)) {
        if (ln.compare(0, 4, "ATOM") == 0) {
            char name[16] = {0};
            if (ln.size() <= 12 || std::sscanf(ln.c_str() + 12, "%15s", name) != 1 || std::strcmp(name, "CA") != 0)
                continue;
            PdbResidue r;
            char res[16] = {0};
            if (ln.size() > 17)
                std::sscanf(ln.c_str() + 17, "%15s", res);
            r.name = res;
            r.chain = ln.size() > 21 ? ln[21] : ' ';
            r.res_seq = 0;
            r.x = r.y = r.z = 0.0f;
            if (ln.size() > 22)
                std::sscanf(ln.c_str() + 22, "%d", &r.res_seq);
            if (ln.size() > 30)
                std::sscanf(ln.c_str() + 30, "%f", &r.x);
            if (ln.size() > 38)
                std::sscanf(ln.c_str() + 38, "%f", &r.y);
            if (ln.size() > 46)
                std::sscanf(ln.c_str() + 46, "%f", &r.z);
            r.chain_index = chains;
            r.type = aa.getAminoAcidIndex(res);
            if (r.type < 0)
                throw "Unknown residue name in PDB file.";
            out.push_back(r);
        } else if (ln.compare(0, 3, "TER") == 0) {
            ++chains;
        } else if (ln.compare(0, 3, "END") == 0) {
            break;
        }
    }
    if (!out.empty() && chains == 0)
        chains = 1;
    if (out.empty())
        throw "No C-alpha records in PDB file.";
    *num_chains = chains;
    return out;
}

PlacedMolecule place_molecule(const std::vector<PdbResidue> &res, int num_chains, bool translate, float px, float py,
                              float pz, float rx, float ry, float rz, float angle, float box)
{
    PlacedMolecule m;
    m.residues = res;
    m.num_chains = num_chains;
    const size_t n = res.size();
    m.pos.resize(3 * n);
    m.rel.resize(3 * n);
    float c[3] = {0, 0, 0};
    for (size_t i = 0; i < n; ++i) {
        m.pos[3 * i] = res[i].x, m.pos[3 * i + 1] = res[i].y, m.pos[3 * i + 2] = res[i].z;
        c[0] += res[i].x, c[1] += res[i].y, c[2] += res[i].z;
    }
    for (int k = 0; k < 3; ++k)
        c[k] = c[k] / (float)n;
    for (size_t i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k)
            m.rel[3 * i + k] = m.pos[3 * i + k] - c[k];
    auto set_position = [&](const float *nc) {
        for (int k = 0; k < 3; ++k)
            m.center[k] = nc[k];
        for (size_t i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k)
                m.pos[3 * i + k] = m.rel[3 * i + k] + m.center[k];
    };
    std::memcpy(m.center, c, sizeof(c));
    const float p[3] = {px, py, pz};
    if (translate) {
        if (px != 0.0f || py != 0.0f || pz != 0.0f) {
            float nc[3];
            for (int k = 0; k < 3; ++k)
                nc[k] = std::fmod(c[k] + p[k], box);
            set_position(nc);
        }
    } else {
        set_position(p);
    }
    if (angle != 0.0f) {
        // Quaternion(angle, axis) normalised, rotateVector in double (src/Quaternion.cpp)
        double ax = rx, ay = ry, az = rz;
        const double mag = std::sqrt(ax * ax + ay * ay + az * az);
        ax /= mag, ay /= mag, az /= mag;
        const double s = std::sin(angle / 2.0), co = std::cos(angle / 2.0);
        double w = co, x = s * ax, y = s * ay, z = s * az;
        const double qm = std::sqrt(w * w + x * x + y * y + z * z);
        w /= qm, x /= qm, y /= qm, z /= qm;
        const double w2 = w * w, x2 = x * x, y2 = y * y, z2 = z * z;
        const double wx = w * x, wy = w * y, wz = w * z, xy = x * y, xz = x * z, yz = y * z;
        for (size_t i = 0; i < n; ++i) {
            const double vx = m.rel[3 * i], vy = m.rel[3 * i + 1], vz = m.rel[3 * i + 2];
            m.rel[3 * i] = (float)(vx * (w2 + x2 - y2 - z2) + (vy * (xy - wz) + vz * (wy + xz)) * 2.0);
            m.rel[3 * i + 1] = (float)((vx * (wz + xy) + vz * (yz - wx)) * 2.0 + vy * (w2 - x2 + y2 - z2));
            m.rel[3 * i + 2] = (float)((vx * (xz - wy) + vy * (yz + wx)) * 2.0 + vz * (w2 - x2 - y2 + z2));
            for (int k = 0; k < 3; ++k)
                m.pos[3 * i + k] = m.center[k] + m.rel[3 * i + k];
        }
    }
    return m;
}

void write_pdb_trace(FILE *out, int n, const float *xyz, const int *types, const int *res_seq, const int *chain,
                     const int *molecule, const AminoAcids &aa, int *atom_counter)
{
    // the three-letter name in capitals, as AminoAcid::getSNAME gives it (src/AminoAcid.cpp:19-25)
    auto sname = [&](int type, char *buf) {
        for (int k = 0; k < 3; ++k)
            buf[k] = (char)std::toupper((unsigned char)aa.data[type].sname[k]);
        buf[3] = 0;
        return buf;
    };
    char nm[4];
    for (int i = 0; i < n; ++i) {
        const char c = (char)(65 + chain[i]);
        if (i > 0 && molecule[i] == molecule[i - 1] && chain[i] != chain[i - 1])
            std::fprintf(out, "TER   %5d      %3s %c%4d \n", *atom_counter, sname(types[i - 1], nm),
                         (char)(65 + chain[i - 1]), res_seq[i - 1]);
        ++*atom_counter;
        std::fprintf(out, "ATOM  %5d CA   %3s %c%4d    %8.3f%8.3f%8.3f%6.2f%6.2f\n", *atom_counter,
                     sname(types[i], nm), c, res_seq[i], xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.0f, 0.0f);
        if (i + 1 == n || molecule[i + 1] != molecule[i])
            std::fprintf(out, "TER   %5d      %3s %c%4d \n", *atom_counter, sname(types[i], nm), c, res_seq[i]);
    }
}

void write_pdb_atoms(FILE *out, const std::vector<PdbResidue> &res, const float *pos, const AminoAcids &aa,
                     int *atom_counter, int chain_base)
{
    const int n = (int)res.size();
    std::vector<int> types(n), seq(n), chain(n), molecule(n, 0);
    for (int i = 0; i < n; ++i) {
        types[i] = res[i].type;
        seq[i] = res[i].res_seq;
        chain[i] = chain_base + res[i].chain_index;
    }
    write_pdb_trace(out, n, pos, types.data(), seq.data(), chain.data(), molecule.data(), aa, atom_counter);
}

void write_sample_pdb(FILE *out, const char *title, float temperature, int sample, double potential, int n,
                      const float *xyz, const int *types, const int *res_seq, const int *chain, const int *molecule,
                      const AminoAcids &aa)
{
    std::fprintf(out, "REMARK simulation: %s \n", title);
    std::fprintf(out, "REMARK temperature: %5.1f \n", (double)temperature);
    std::fprintf(out, "REMARK sample: %d \n", sample);
    std::fprintf(out, "REMARK potential: %0.10f \n", (double)(float)potential);
    int counter = 0;
    write_pdb_trace(out, n, xyz, types, res_seq, chain, molecule, aa, &counter);
    std::fprintf(out, "END \n");
}

}  // namespace cgppd

extern "C" int cgppd_pdb_read(const char *path, const AminoAcids *a, int capacity, float *xyz, int *types,
                              char *chain_ids, int *res_seq, int *chain_index, int *num_chains)
{
    if (!path || !a)
        return cgppd_fail("cgppd_pdb_read: path and residue table are required");
    std::vector<cgppd::PdbResidue> res;
    int chains = 0;
    try {
        res = cgppd::read_pdb(path, *a, &chains);
    } catch (const char *msg) {
        return cgppd_fail(msg);
    }
    const int n = (int)res.size();
    if (capacity >= n) {
        for (int i = 0; i < n; ++i) {
            if (xyz) {
                xyz[3 * i] = res[i].x;
                xyz[3 * i + 1] = res[i].y;
                xyz[3 * i + 2] = res[i].z;
            }
            if (types)
                types[i] = res[i].type;
            if (chain_ids)
                chain_ids[i] = res[i].chain;
            if (res_seq)
                res_seq[i] = res[i].res_seq;
            if (chain_index)
                chain_index[i] = res[i].chain_index;
        }
    }
    if (num_chains)
        *num_chains = chains;
    return n;
}

extern "C" int cgppd_pdb_write_sample(const char *path, const AminoAcids *a, const char *title, float temperature,
                                      int sample, double potential, int n, const float *xyz, const int *types,
                                      const int *res_seq, const int *chain, const int *molecule)
{
    if (!path || !a || !title || n < 0 || (n > 0 && (!xyz || !types || !res_seq || !chain || !molecule)))
        return cgppd_fail("cgppd_pdb_write_sample: path, table, title and n residue records are required");
    for (int i = 0; i < n; ++i)
        if (types[i] < 0 || types[i] >= 20 || chain[i] < 0 || chain[i] > 25)
            return cgppd_fail("cgppd_pdb_write_sample: residue type outside 0..19 or chain outside A..Z");
    FILE *f = std::fopen(path, "w");
    if (!f)
        return cgppd_fail("cgppd_pdb_write_sample: cannot open the output file");
    cgppd::write_sample_pdb(f, title, temperature, sample, potential, n, xyz, types, res_seq, chain, molecule, *a);
    std::fclose(f);
    return 0;
}
