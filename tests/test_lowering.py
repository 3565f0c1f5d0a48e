"""Host lowering of Density / Current / matrix operators to the device term
form, checked on the CPU against the reference's golden outputs (through a
numpy evaluation of the term form) and against the oracle."""

import numpy as np
import pytest

from golden_io import load, csr
from oracle import kpm_oracle as ko
from kwant_gb300 import operator as kop
from kwant_gb300.system import LatticeSystem


def evaluate_host(low, bra, ket):
    """Numpy evaluation of a lowered operator's term form: per term the
    bra coefficient sum_j conj(b_j) bra[col_j], then conj(coef) ket[row]
    accumulated into the term's output slot."""
    bra = np.asarray(bra, complex)
    ket = np.asarray(ket, complex)
    seg = np.repeat(np.arange(low.num_terms), np.diff(low.bra_ptr))
    coef = np.zeros(low.num_terms, complex)
    np.add.at(coef, seg, np.conj(low.bra_val) * bra[low.bra_col])
    contrib = np.conj(coef) * ket[low.term_row]
    out = np.zeros(low.num_outputs, complex)
    tchunk = np.repeat(np.arange(low.num_chunks), np.diff(low.chunk_ptr))
    np.add.at(out, low.chunk_out[tchunk], contrib)
    return out


def _rashba_system(g):
    ham = csr(g)
    n = ham.shape[0]
    return LatticeSystem(ham, [(0, 2, 0), (n // 2, 0, n)], g['positions'])


def test_density_local_matrix_onsite():
    g = load('rashba_ops')
    syst = _rashba_system(g)
    sz = np.diag([1.0, -1.0])
    d = kop.Density(syst, onsite=sz, where=list(g['where_sites']))
    low = kop.lower(d)
    got = evaluate_host(low, g['bra'], g['ket'])
    np.testing.assert_allclose(got, g['dens_loc_call'], rtol=0, atol=1e-12)


def test_density_summed():
    g = load('rashba_ops')
    syst = _rashba_system(g)
    d = kop.Density(syst, onsite=np.diag([1.0, -1.0]), sum=True)
    low = kop.lower(d)
    assert low.num_outputs == 1 and low.scalar
    got = evaluate_host(low, g['bra'], g['ket'])[0]
    assert abs(got - g['dens_sz_call']) < 1e-10


def test_current_lowering():
    g = load('rashba_ops')
    syst = _rashba_system(g)
    hw = [tuple(x) for x in g['hop_where']]
    c = kop.Current(syst, onsite=np.diag([1.0, -1.0]), where=hw)
    low = kop.lower(c)
    got = evaluate_host(low, g['bra'], g['ket'])
    np.testing.assert_allclose(got, g['cur_call'], rtol=0, atol=1e-12)


def test_act_matrices():
    g = load('rashba_ops')
    syst = _rashba_system(g)
    n = syst.num_orbitals
    sz = np.diag([1.0, -1.0])
    d = kop.Density(syst, onsite=sz, where=list(g['where_sites']))
    np.testing.assert_allclose(kop.act_matrix(d, n) @ g['ket'],
                               g['dens_loc_act'], atol=1e-12)
    hw = [tuple(x) for x in g['hop_where']]
    c = kop.Current(syst, onsite=sz, where=hw)
    np.testing.assert_allclose(kop.act_matrix(c, n) @ g['ket'],
                               g['cur_act'], atol=1e-12)


def test_chain_current_scalar_sites():
    g = load('chain_current')
    ham = csr(g)
    n = ham.shape[0]
    syst = LatticeSystem(ham, [(0, 1, 0), (n, 0, n)],
                         np.arange(n, dtype=float)[:, None])
    where = [tuple(w) for w in g['where']]
    c = kop.Current(syst, where=where)
    rs = np.random.RandomState(3)
    bra = rs.randn(n) + 1j * rs.randn(n)
    ket = rs.randn(n) + 1j * rs.randn(n)
    blocks = [ham[a:a + 1, b:b + 1].toarray() for a, b in where]
    ref = ko.current_matels(bra, ket, [(0, 1, 0), (n, 0, n)], where, blocks,
                            np.eye(1))
    np.testing.assert_allclose(evaluate_host(kop.lower(c), bra, ket), ref,
                               atol=1e-12)


def test_matrix_operator_lowering():
    rs = np.random.RandomState(5)
    O = rs.randn(12, 12) + 1j * rs.randn(12, 12)
    O[np.abs(O) < 0.8] = 0
    bra = rs.randn(12) + 1j * rs.randn(12)
    ket = rs.randn(12) + 1j * rs.randn(12)
    low = kop.lower_matrix(O)
    assert low.scalar
    got = evaluate_host(low, bra, ket)[0]
    assert abs(got - np.vdot(bra, O @ ket)) < 1e-12


def test_sum_chunking_large():
    n = 1000
    sr = [(0, 1, 0), (n, 0, n)]
    low = kop.lower_density(sr, np.arange(n), np.eye(1), sum_=True)
    assert low.num_chunks == (n + kop.SUM_CHUNK - 1) // kop.SUM_CHUNK
    rs = np.random.RandomState(1)
    v = rs.randn(n) + 1j * rs.randn(n)
    assert abs(evaluate_host(low, v, v)[0] - np.vdot(v, v)) < 1e-10


def test_where_validation():
    g = load('rashba_ops')
    syst = _rashba_system(g)
    with pytest.raises(ValueError):
        kop.Density(syst, where=[10 ** 6])
    with pytest.raises(ValueError):
        kop.Current(syst, where=[(0, 35)])
    with pytest.raises(ValueError):
        kop.Density(syst, onsite=np.array([[1, 1j], [0, 1]]))
