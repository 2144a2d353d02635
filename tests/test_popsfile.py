"""POPSFILE version 4 (Popsfile.F90): the writer reproduces the record bytes
of POPSFILEs that NECI wrote in its own test suite, the header namelist is
read as ReadPopsHeadv4 reads it, and a binary POPSFILE restarts a run bit for
bit (through the CPU oracle here; through the engine in test_gpu_parity)."""
from __future__ import annotations

import hashlib
from pathlib import Path

import numpy as np
import pytest

from neci_stable_gb300 import capi, popsfile
from neci_stable_gb300.popsfile import PopsHeader

GOLDEN = Path(__file__).parent / "golden"


def load(name):
    d = np.load(GOLDEN / name)
    return str(d["header"]), d["rows"], bool(d["binary"]), str(d["sha256"])


@pytest.mark.parametrize("name", ["pops_text_li2.npz", "pops_bin_ne.npz", "pops_bin_beh_dneci.npz"])
def test_writer_reproduces_neci_record_bytes(name):
    head, rows, binary, sha = load(name)
    h = popsfile.parse_header(head)
    W, L = h.nifd + 1, h.lenof_sign
    assert rows.shape == (h.totwalk, W + L + 1)
    data = popsfile.records_binary(rows, W, L) if binary else popsfile.records_text(rows, W, L).encode()
    assert hashlib.sha256(data).hexdigest() == sha
    back = (popsfile.parse_records_binary(data, W, L) if binary
            else popsfile.parse_records_text(data.decode(), W, L))
    assert np.array_equal(back, rows)


def test_header_values_as_neci_wrote_them():
    h = popsfile.parse_header(load("pops_text_li2.npz")[0])
    assert (h.nel, h.lenof_sign, h.nifd, h.totwalk, h.cyc) == (6, 1, 0, 439, 1000)
    assert h.tau == 0.029379531779 and h.p_singles == 0.301798861504 and h.p_parallel == 0.112571190307
    assert h.gamma_sing == 10.2723163115 and h.gamma_opp == 21.0894310328 and h.gamma_par == 2.67521442660
    assert h.max_death_cpt == 11.6940420807 and h.tot_imag_time == 22.136683845193
    assert h.shift == [0.0] and h.sum_noat_hf == [145592.82685607419] and h.sum_enum == [-35154.849886457880]
    assert h.balance_blocks == 400 and h.walkers_on_nodes == [102, 9, 220, 108]
    assert len(h.random_hash) == 20 and h.random_hash[0] == 14677 and not h.auto_adaptive_shift
    # a header another compiler wrote (E-format list-directed reals), two replicas
    d = popsfile.parse_header(load("pops_bin_beh_dneci.npz")[0])
    assert d.lenof_sign == 2 and d.nel == 3 and d.totwalk == 588
    assert d.shift[0] == pytest.approx(-3.762213846960396e-2, rel=0, abs=0)


@pytest.mark.parametrize("name", ["pops_text_li2.npz", "pops_bin_ne.npz", "pops_bin_beh_dneci.npz"])
def test_header_round_trip(name):
    h = popsfile.parse_header(load(name)[0])
    h2 = popsfile.parse_header(popsfile.header_text(h))
    for f in ("nel", "lenof_sign", "nifd", "totwalk", "cyc", "tau", "p_singles", "p_parallel", "shift",
              "sum_noat_hf", "sum_enum", "gamma_sing", "gamma_opp", "gamma_par", "max_death_cpt", "random_hash",
              "walkers_on_nodes", "tot_imag_time"):
        a, b = getattr(h, f), getattr(h2, f)
        if f in ("shift", "sum_noat_hf", "sum_enum"):
            np.testing.assert_allclose(a, b, rtol=1e-15, atol=0, err_msg=f)
        else:
            assert a == b, f


def test_fortran_g_editing():
    g = popsfile.fortran_g
    assert g(0.0) == "   0.0000000000000000     "
    assert g(145592.82685607419) == "   145592.82685607419     "
    assert g(-35154.849886457880) == "  -35154.849886457880     "
    assert g(1.0) == "   1.0000000000000000     "
    assert len(g(-3.762213846960396e-2)) == 26 and float(g(-3.762213846960396e-2)) == -3.762213846960396e-2


@pytest.mark.parametrize("binary", [True, False])
def test_restart_from_popsfile_continues_the_run(tmp_path, binary):
    """Write after 8 iterations, read back into a fresh oracle, run 6 more:
    identical to running 14 (binary), or within the text form's 8 decimals."""
    from helpers import canonical, molecule
    from oracle.oracle import Oracle
    spec = molecule(12, 6)
    W, L = spec.W, spec.lenof_sign

    def fresh():
        from neci_stable_gb300.systems import encode_det, make_rows
        o = Oracle(spec, 100_000, 200_000)
        ref = encode_det(spec.reference, spec.nifd)
        o.upload(make_rows(ref[None], np.array([[40.0]]), np.array([1 << 13])))
        return o

    par = lambda it: capi.default_params(tau=0.02, seed=3, iter=it)  # noqa: E731
    a = fresh()
    for it in range(1, 9):
        a.iterate(par(it))
    rows = a.download()[0]
    hdr = PopsHeader(nel=spec.nel, lenof_sign=L, nifd=spec.nifd, cyc=8, tau=0.02, p_singles=spec.p_singles,
                     p_parallel=spec.p_parallel, p_doubles=1.0 - spec.p_singles,
                     random_hash=list(map(int, spec.random_hash2)))
    popsfile.write_popsfile(tmp_path / "POPSFILE", hdr, rows, binary=binary)
    h, back = popsfile.read_popsfile(tmp_path / "POPSFILE")
    assert h.totwalk == back.shape[0] and h.cyc == 8
    b = fresh()
    b.upload(back)
    for it in range(9, 15):
        a.iterate(par(it))
        b.iterate(par(it))
    ra, rb = canonical(a.download()[0], W), canonical(b.download()[0], W)
    if binary:
        assert np.array_equal(ra[:, :W + L], rb[:, :W + L])
    else:
        assert ra.shape[0] > 0 and rb.shape[0] > 0
        np.testing.assert_allclose(np.abs(rb[:, W:W + L].view(np.float64)).sum(),
                                   np.abs(ra[:, W:W + L].view(np.float64)).sum(), rtol=0.05)
