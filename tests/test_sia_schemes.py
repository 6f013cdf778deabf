"""SIA composition tables (CPU): the GPU integrator's operator sequences
(tupan_gb300.integrator.sia.palindrome) equal the CPU restatement's
(oracle.integrators.sia_sequence) and the reference's written-out
propagators (tupan/integrator/sia.py:300-961), and the method list is the
reference's 48 names (sia.py:969-985)."""
import pytest

pytest.importorskip("torch")

from oracle.integrators import SIA_COEFS, sia_sequence  # noqa: E402


def sia_module():
    from tupan_gb300.integrator import sia
    return sia


def test_gpu_and_oracle_tables_agree():
    sia = sia_module()
    assert sia.COEFS == SIA_COEFS
    for name, (first, second) in sia.COEFS.items():
        assert sia.palindrome(first, second) == sia_sequence(first, second), name


def test_sequences_match_reference_listings():
    """kdk of SIA44 and dkd of SIA46, written out as in sia.py: operator 0
    is the kick (kdk) or drift (dkd) and takes the second coefficient list."""
    sia = sia_module()
    d, k = sia.COEFS["sia44"]          # kdk: d, k = coefs
    want = [(0, k[0]), (1, d[0]), (0, k[1]), (1, d[1]), (0, k[2]),
            (1, d[1]), (0, k[1]), (1, d[0]), (0, k[0])]
    assert sia.palindrome(*sia.COEFS["sia44"]) == want
    k, d = sia.COEFS["sia46"]          # dkd: k, d = coefs
    want = [(0, d[0]), (1, k[0]), (0, d[1]), (1, k[1]), (0, d[2]), (1, k[2]), (0, d[3]),
            (1, k[2]), (0, d[2]), (1, k[1]), (0, d[1]), (1, k[0]), (0, d[0])]
    assert sia.palindrome(*sia.COEFS["sia46"]) == want


def test_sequences_are_symmetric_and_consistent():
    sia = sia_module()
    for name, (first, second) in sia.COEFS.items():
        seq = sia.palindrome(first, second)
        assert seq == seq[::-1], name
        # each operator's coefficients over the whole step sum to 1
        tot0 = sum(c for op, c in seq if op == 0)
        tot1 = sum(c for op, c in seq if op == 1)
        assert abs(tot0 - 1) < 1e-12 and abs(tot1 - 1) < 1e-12, (name, tot0, tot1)


def test_method_names_are_the_references():
    sia = sia_module()
    want = {"sia%s%s.%s" % (o, m, f) for o in ("21", "22", "43", "44", "45", "46", "67", "69")
            for m in "sah" for f in ("dkd", "kdk")}
    assert set(sia.SIA.PROVIDED_METHODS) == want and len(want) == 48
