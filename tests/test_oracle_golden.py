"""The CPU oracle reproduces SEAL's own outputs stored in tests/golden/ckks_n4096.npz."""
import numpy as np

from oracle import pyoracle as po
from tests.golden_data import load

G = load()
QS = [int(q) for q in G["moduli"]]
OC = po.OracleContext(int(G["log_n"]), QS)


def test_ntt_matches_seal():
    assert np.array_equal(OC.ntt(G["ntt_in"], 0, 3), G["ntt_out"])


def test_multiply_relin_rescale():
    mul3 = OC.multiply(G["ct_a"], G["ct_b"])
    assert np.array_equal(mul3, G["mul3"])
    relin = OC.relinearize(mul3, G["relin_key"])
    assert np.array_equal(relin, G["relin"])
    assert np.array_equal(OC.rescale(relin), G["rescaled"])


def test_rotations_and_conjugation():
    e1, em3, e0 = [int(e) for e in G["galois_elts"]]
    assert e1 == po.galois_elt_from_step(12, 1) and em3 == po.galois_elt_from_step(12, -3)
    assert np.array_equal(OC.apply_galois(G["ct_a"], e1, G["galois_key_1"]), G["rot1"])
    assert np.array_equal(OC.apply_galois(G["ct_a"], em3, G["galois_key_m3"]), G["rotm3"])
    assert np.array_equal(OC.apply_galois(G["ct_a"], e0, G["galois_key_conj"]), G["conj"])
    low = np.ascontiguousarray(G["ct_a"][:, :1])
    assert np.array_equal(OC.apply_galois(low, e1, G["galois_key_1"]), G["rot1_low"])


def test_multiply_plain():
    assert np.array_equal(OC.multiply_plain(G["ct_a"], G["pt"]), G["mulplain"])
