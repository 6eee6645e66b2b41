"""The native library builds, loads and exports the declared ABI (no GPU calls)."""
import ctypes

import numpy as np
import pytest

import cgppd_gb300
from helpers import header_functions, write_amino_acid_file, write_lj_file


@pytest.fixture(scope="module")
def L():
    cgppd_gb300.build()
    return cgppd_gb300.lib()


def test_exports_every_declared_symbol(L):
    names = header_functions()
    assert "CUDA_EonDevice" in names and "CUDA_EonDevice_async" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_amino_acids_layout_matches_reference(L):
    # LJpotentials sits after AminoAcid data[20] (48 bytes each, vtable pointer first),
    # as in src/AminoAcids.h:12-13 compiled with the Itanium C++ ABI.
    assert L.cgppd_aminoacids_lj_offset() == 960
    assert L.cgppd_aminoacids_sizeof() == 2568


def test_loaders_read_reference_formats(L, refdata, tmp_path):
    aa_path, lj_path = tmp_path / "AminoAcids", tmp_path / "pairs"
    write_amino_acid_file(str(aa_path), refdata["amino_acids"])
    write_lj_file(str(lj_path), refdata["amino_acids"], refdata["lj_table"])
    a = L.cgppd_aminoacids_create()
    try:
        assert L.cgppd_aminoacids_load(a, str(aa_path).encode(), str(lj_path).encode()) == 0
        t = (ctypes.c_float * 400)()
        L.cgppd_aminoacids_get_table(a, t)
        got = np.array(t[:], np.float32).reshape(20, 20)
        assert np.allclose(got, np.array(refdata["lj_table"], np.float32), atol=1e-6)
        assert np.allclose(got, got.T)
        # getAminoAcidIndex: 3-letter (any case), 1-letter, full name, unknown -> -1
        assert L.cgppd_aminoacids_index(a, b"TYR") == 16
        assert L.cgppd_aminoacids_index(a, b"tyr") == 16
        assert L.cgppd_aminoacids_index(a, b"Y") == 16
        assert L.cgppd_aminoacids_index(a, b"Tyrosine") == 16
        assert L.cgppd_aminoacids_index(a, b"XYZ") == -1
        assert L.cgppd_aminoacids_index(a, b"") == -1
    finally:
        L.cgppd_aminoacids_destroy(a)


def test_missing_file_is_reported(L, tmp_path):
    a = L.cgppd_aminoacids_create()
    try:
        assert L.cgppd_aminoacids_load(a, str(tmp_path / "nope").encode(), b"nope") != 0
    finally:
        L.cgppd_aminoacids_destroy(a)
