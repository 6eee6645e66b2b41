// amino_acids.h -- residue-type parameters and the 20x20 contact table.
//
// The drop-in C ABI takes `AminoAcids*` (src/cudaExterns.h:19-20) and reads the
// contact table straight out of the caller's object, so this class keeps the
// reference's member order and types (src/AminoAcid.h:12-24, src/AminoAcids.h:7-27):
// AminoAcid has a virtual destructor (one vtable pointer) and AminoAcids is
// `AminoAcid data[20]; float LJpotentials[20][20]; bool clean;`.  The offsets are
// pinned by static_asserts below and by a test against the reference's own header.
#pragma once

#include <cstddef>

class AminoAcid {
public:
    AminoAcid();
    virtual ~AminoAcid();
    char name[20];
    char sname[4];
    char shortSymbol;
    float vanderWaalRadius;
    float electrostaticCharge;
    int index;
    char *getSNAME() { return sname; }
};

class AminoAcids {
public:
    AminoAcids();
    ~AminoAcids();
    AminoAcid data[20];
    float LJpotentials[20][20];
    bool clean;

    // Same text formats as the reference loaders (src/AminoAcids.cpp:29-138).
    void init(const char *aminoAcidFile, const char *ljFile);
    bool loadAminoAcidData(const char *path);
    bool loadLJPotentialData(const char *path);
    // Index lookup by 3-letter, 1-letter or full name; -1 when unknown
    // (src/AminoAcids.cpp:145-181).
    int getAminoAcidIndex(const char *name) const;
    AminoAcid get(int i) const { return data[i]; }
    float getLJp(int a, int b) const { return LJpotentials[a][b]; }
};

// AminoAcids is not standard-layout (AminoAcid is polymorphic), so offsetof is only
// conditionally supported; both compilers used here (g++, nvcc's EDG front end) give
// the Itanium-ABI offsets, which are what the reference build has.
#if defined(__GNUC__)
#pragma GCC diagnostic push
#pragma GCC diagnostic ignored "-Winvalid-offsetof"
#endif
#ifdef __NVCC__
#pragma nv_diag_suppress 1427
#endif
static_assert(sizeof(AminoAcid) == 48, "AminoAcid layout must match the reference");
static_assert(offsetof(AminoAcids, LJpotentials) == 960, "LJpotentials offset must match the reference");
#if defined(__GNUC__)
#pragma GCC diagnostic pop
#endif
