"""The coded-link simulation on the device: random bits against a NumPy
restatement of Philox-4x32-10, the encoder against the host encoders and
H c = 0, the mapping and noise against the host, one batch's error counts
against the oracle on the same symbols (exactly), the error-rate loop, and
GMI / NGMI against the reference's values."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from commkit_gb300 import workloads as W
from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu

M32 = (1 << 32) - 1


def philox_np(counters: np.ndarray, stream: int, seed: int) -> np.ndarray:
    """Philox-4x32-10 (Salmon et al., SC 2011) of 64-bit counters: (n, 4) uint32."""
    c = np.stack([counters & M32, counters >> 32, np.full_like(counters, stream & M32),
                  np.full_like(counters, stream >> 32)], axis=1).astype(np.uint64)  # fmt: skip
    k0, k1 = np.uint64(seed & M32), np.uint64(seed >> 32)
    for _ in range(10):
        p0 = np.uint64(0xD2511F53) * c[:, 0]
        p1 = np.uint64(0xCD9E8D57) * c[:, 2]
        hi0, lo0, hi1, lo1 = p0 >> np.uint64(32), p0 & np.uint64(M32), p1 >> np.uint64(32), p1 & np.uint64(M32)
        c = np.stack([hi1 ^ c[:, 1] ^ k0, lo1, hi0 ^ c[:, 3] ^ k1, lo0], axis=1)
        k0, k1 = (k0 + np.uint64(0x9E3779B9)) & np.uint64(M32), (k1 + np.uint64(0xBB67AE85)) & np.uint64(M32)
    return c.astype(np.uint32)


def bits_np(count: int, seed: int, stream: int) -> np.ndarray:
    words = philox_np(np.arange((count + 127) // 128, dtype=np.uint64), stream, seed)
    return ((words[:, :, None] >> np.arange(32, dtype=np.uint32)) & 1).reshape(-1)[:count].astype(np.int8)


@pytest.fixture(scope="module")
def torch_dev():
    import torch

    return torch, torch.device("cuda", 0)


def test_random_bits_match_philox(torch_dev):
    torch, dev = torch_dev
    from commkit_gb300 import _lib

    for count, seed, stream in ((1000, 7, 3), (128 * 37 + 5, 2**62 + 11, 2**40 + 1)):
        out = torch.empty(count, dtype=torch.int8, device=dev)
        st = torch.cuda.current_stream().cuda_stream
        _lib.check(_lib.lib().ck_random_bits(out.data_ptr(), count, seed, stream, st), "bits")
        np.testing.assert_array_equal(out.cpu().numpy(), bits_np(count, seed, stream))


def _codes(ck):
    g = dict(np.load(GOLDEN / "ldpc_golden.npz"))
    d = dict(np.load(GOLDEN / "dvbs2_normal.npz"))
    out = {n: ck.LDPCCode.quasi_cyclic(W.CODES[n].base(), lifting=W.CODES[n].z) for n in ("A", "C")}
    out["dvbs2n"] = ck.LDPCCode(d["dvbs2n_checks"], d["dvbs2n_variables"], int(d["dvbs2n_m"]), int(d["dvbs2n_N"]))
    out["pon"] = ck.LDPCCode(g["pon_checks"], g["pon_variables"], int(g["pon_m"]), int(g["pon_N"]),
                             int(g["pon_N"]) - int(g["pon_n"]))  # fmt: skip
    return out


def test_encoder_against_host(torch_dev):
    """Accumulators of stride Z (codes A, C: one thread per chain), stride 1
    (DVB-S2: block scans), and an inverse (PON, punctured): systematic, every
    check satisfied, and equal to the host encoders where there is one."""
    import commkit_gb300 as ck

    torch, dev = torch_dev
    rng = np.random.default_rng(3)
    for name, code in _codes(ck).items():
        B = 5
        info = rng.integers(0, 2, size=(B, code.k), dtype=np.int8)
        words = ck.encode(torch.from_numpy(info.reshape(-1)).to(dev), code=code).cpu().numpy().reshape(B, code.n)
        np.testing.assert_array_equal(words[:, : code.k], info)
        full = np.zeros((B, code.num_variables), np.int64)
        full[:, : code.n] = words
        if code.punctured:  # the punctured parity bits: encode again with room for them
            e = code._encoder
            assert e.inverse is not None
        else:
            syn = np.zeros((B, code.num_checks), np.int64)
            np.add.at(syn.T, code.checks, full[:, code.variables].T)
            assert not np.any(syn % 2), name
        if name in ("A", "C"):
            np.testing.assert_array_equal(words, W.encode_qc(W.CODES[name].base(), W.CODES[name].z, info))
        if name == "dvbs2n":
            np.testing.assert_array_equal(words, W.encode_accumulate(code.checks, code.variables,
                                                                     code.num_checks, code.k, info))  # fmt: skip
    # PON's transmitted bits leave its punctured parity bits out: decoding
    # clean LLRs of them recovers the information and satisfies every check.
    code = _codes(ck)["pon"]
    info = rng.integers(0, 2, size=(3, code.k), dtype=np.int8)
    w = ck.encode(torch.from_numpy(info).to(dev), code=code).float()
    res = ck.decode(4.0 - 8.0 * w, code=code)
    assert bool(res.valid.all())
    np.testing.assert_array_equal(res.bits.cpu().numpy().reshape(3, -1), info)


def test_map_and_noise(torch_dev):
    import commkit_gb300 as ck
    from commkit_gb300 import _lib
    from commkit_gb300.mapping import _packed

    torch, dev = torch_dev
    c = ck.Constellation.qam(16)
    by_label = np.empty(16, np.complex64)
    by_label[_packed(c.bit_labels)] = c.points.astype(np.complex64)
    pts = torch.from_numpy(by_label).to(dev)
    n = 50_000
    bits = torch.from_numpy(np.random.default_rng(1).integers(0, 2, 4 * n, dtype=np.int8)).to(dev)
    out = torch.empty(n, dtype=torch.complex64, device=dev)
    st = torch.cuda.current_stream().cuda_stream
    lib = _lib.lib()
    _lib.check(lib.ck_map_awgn(bits.data_ptr(), n, 4, pts.data_ptr(), 0.0, 0.0, 1, 2, out.data_ptr(), st), "map")
    labels = (bits.cpu().numpy().reshape(n, 4).astype(np.int64) << np.arange(3, -1, -1)).sum(1)
    np.testing.assert_array_equal(out.cpu().numpy(), by_label[labels])
    s = 0.3
    _lib.check(lib.ck_map_awgn(bits.data_ptr(), n, 4, pts.data_ptr(), s, s, 9, 5, out.data_ptr(), st), "awgn")
    noise = out.cpu().numpy().astype(np.complex128) - by_label[labels]
    r = philox_np(np.arange(n, dtype=np.uint64), 5, 9)
    u1 = ((r[:, 0] >> 8).astype(np.float64) + 0.5) * 2.0**-24
    u2 = ((r[:, 1] >> 8).astype(np.float64) + 0.5) * 2.0**-24
    rad = np.sqrt(-2.0 * np.log(u1))
    want = s * rad * (np.cos(2 * np.pi * u2) + 1j * np.sin(2 * np.pi * u2))
    np.testing.assert_allclose(noise, want, rtol=0, atol=2e-6)
    assert abs(noise.real.mean()) < 0.01 and abs(noise.real.std() - s) < 0.01 and abs(noise.imag.std() - s) < 0.01


@pytest.mark.parametrize("name, order, esn0", [("A", 4, 1.5), ("B", 16, 10.0), ("B", 8, 8.0), ("tiny", 8, 4.0)])
def test_batch_counts_match_oracle(torch_dev, name, order, esn0):
    """One batch on the device; the oracle demaps the same symbols, decodes
    and counts: the counts agree exactly.  8-PSK takes the M-point demapper;
    the tiny code's 40 x 40 bits do not fill whole 8-PSK symbols, so the
    record ends in filler bits."""
    import commkit_gb300 as ck
    from commkit_gb300.performance import LinkBatch
    from tests.test_constellations import oracle_llr

    torch, dev = torch_dev
    if name == "tiny":
        code = ck.LDPCCode.quasi_cyclic(W.dual_diagonal_base(3, 8, 5, (2,) * 5, seed=3), lifting=5)
        assert (40 * code.n) % 3
    else:
        code = ck.LDPCCode.quasi_cyclic(W.CODES[name].base(), lifting=W.CODES[name].z)
    c = ck.Constellation.psk(8) if order == 8 else ck.Constellation.qam(order)
    link = LinkBatch(code, c, ck.MinSum(max_iterations=20), 40, dev, seed=1234)
    nv = c.power() / 10 ** (esn0 / 10)
    link.run(nv, stream_id=3)
    got = link.counts.cpu().numpy()
    info = link.info.cpu().numpy()
    words = link.words.cpu().numpy()
    sym = link.symbols.cpu().numpy()
    llr = oracle_llr(c, sym, nv, "maxlog").reshape(-1)[: 40 * code.n].reshape(40, code.n)
    np.testing.assert_array_equal(llr, link.llrs.cpu().numpy())
    row_ptr, cols, _ = code._schedule
    bits, post, valid, iters = oracle.decode(llr, (row_ptr, cols, code.num_variables), k=code.k, max_iterations=20)
    wrong = bits != info
    bw = wrong.any(axis=1)
    want = [40, wrong.sum(), bw.sum(), ((llr < 0) != (words != 0)).sum(), (~valid).sum(), (bw & valid).sum(),
            iters.sum()]  # fmt: skip
    np.testing.assert_array_equal(got, want)
    assert 0 < got[3] < 40 * code.n  # the channel made errors


def test_error_rate_curve(torch_dev):
    import commkit_gb300 as ck

    torch, dev = torch_dev
    code = ck.LDPCCode.quasi_cyclic(W.CODES["A"].base(), lifting=W.CODES["A"].z)
    c = ck.Constellation.qam(4)
    kw = dict(constellation=c, esn0_db=[-1.0, 1.0, 2.5], method=ck.MinSum(max_iterations=20),
              min_block_errors=30, max_blocks=2000, rng=5)  # fmt: skip
    a = ck.error_rate_curve(code, **kw)
    b = ck.error_rate_curve(code, **kw)
    for f in ("num_blocks", "bit_errors", "block_errors", "pre_fec_bit_errors", "total_iterations"):
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f))  # reproducible for a seed
    assert a.fer[0] > a.fer[1] > a.fer[2] and a.pre_fec_ber[0] > a.pre_fec_ber[2]
    assert np.all((a.block_errors >= 30) | (a.num_blocks == 2000))
    assert np.all(a.undetected_errors <= a.block_errors) and a.k == code.k and a.n == code.n
    # BPSK (real) through the M-point path: pre-FEC BER near Q(sqrt(2 Es/N0)).
    pam = ck.error_rate_curve(code, constellation=ck.Constellation.psk(2), esn0_db=[0.0], min_block_errors=10**9,
                              max_blocks=400, rng=1)  # fmt: skip
    from math import erfc, sqrt

    assert abs(pam.pre_fec_ber[0] - 0.5 * erfc(sqrt(1.0))) < 0.003


@pytest.mark.parametrize("name", ["q16", "p8", "q64s"])
def test_gmi_matches_reference(torch_dev, name):
    import commkit_gb300 as ck

    torch, dev = torch_dev
    g = dict(np.load(GOLDEN / "gmi_golden.npz"))
    c = {"q16": ck.Constellation.qam(16), "p8": ck.Constellation.psk(8),
         "q64s": ck.Constellation.qam(64).shaped(entropy=5.0)}[name]  # fmt: skip
    L, b = torch.from_numpy(g[f"{name}_llrs"]).to(dev), torch.from_numpy(g[f"{name}_bits"]).to(dev)
    np.testing.assert_allclose(ck.gmi(L, b, constellation=c), g[f"{name}_gmi2"], rtol=1e-6)
    np.testing.assert_allclose(ck.ngmi(L, b, constellation=c), g[f"{name}_ngmi2"], rtol=1e-6)
    assert ck.gmi(L[0], b[0], constellation=c) == pytest.approx(float(g[f"{name}_gmi1"]), rel=1e-6)
    assert ck.gmi(L[0], b[0], constellation=c, num_skip_symbols=5) == pytest.approx(float(g[f"{name}_gmi1_skip"]),
                                                                                    rel=1e-6)  # fmt: skip
