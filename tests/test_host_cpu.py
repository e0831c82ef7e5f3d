"""Host side of the drop-in on CPU (no GPU calls): the event reader and the
reference-format writer of libhbt_host.so, checked on the golden cases."""
import ctypes
import os
import tarfile
import zlib

import numpy as np
import pytest

import oracle_lib
import parity
from hadronic_afterburner_toolkit_gb300 import build, engine, synth

CASES = sorted(d for d in os.listdir(oracle_lib.GOLDEN)
               if os.path.exists(os.path.join(oracle_lib.GOLDEN, d, "parameters.dat")))
_PD = ctypes.POINTER(ctypes.c_double)
_PU = ctypes.POINTER(ctypes.c_uint64)


@pytest.fixture(scope="module")
def host():
    build.build_gpu()
    lib = build.build_host()
    L = ctypes.CDLL(lib)
    L.hbt_host_scan_buffers.restype = ctypes.c_int
    L.hbt_host_scan_buffers.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32,
                                        ctypes.POINTER(ctypes.c_int32),
                                        ctypes.POINTER(ctypes.c_int64),
                                        ctypes.POINTER(ctypes.c_int32),
                                        ctypes.POINTER(ctypes.c_int64)]
    L.hbt_host_write.restype = ctypes.c_int
    L.hbt_host_write.argtypes = [ctypes.POINTER(engine.HbtParams), ctypes.c_char_p,
                                 ctypes.c_int32] + [_PD] * 10 + [_PU] * 4
    return L


def _stage(name, tmp, root=oracle_lib.GOLDEN):
    src = os.path.join(root, name)
    res = os.path.join(tmp, "results")
    os.makedirs(res, exist_ok=True)
    for fn in os.listdir(src):
        if (fn.endswith(".gz") and fn != "outputs.tar.gz") or fn.endswith(".DAT"):
            os.symlink(os.path.join(src, fn), os.path.join(res, fn))
    return os.path.join(src, "parameters.dat"), res


@pytest.mark.parametrize("name", CASES)
def test_reader_buffers_match_reference_rule(host, name, tmp_path):
    _check_buffers(host, name, str(tmp_path), oracle_lib.GOLDEN)


def _check_buffers(host, name, tmp, root):
    """The reader's buffers (events and particles of the analysed species,
    same-event and mixed-event) against the reference's buffering rule as
    the oracle restates it (whole events until the count reaches
    event_buffer_size)."""
    pfile, res = _stage(name, tmp, root)
    cap = 4096
    nev = (ctypes.c_int32 * cap)()
    npart = (ctypes.c_int64 * cap)()
    mnev = (ctypes.c_int32 * cap)()
    mpart = (ctypes.c_int64 * cap)()
    nb = host.hbt_host_scan_buffers(pfile.encode(), res.encode(), cap, nev, npart, mnev, mpart)
    assert nb > 0
    prm, ev, mixed = oracle_lib.golden_case(name, root)
    size = int(prm["event_buffer_size"])
    mon = int(prm["particle_monval"])
    want = oracle_lib.buffer_ranges(ev.multiplicities(), size)
    # the reader sees one trailing empty buffer when the last buffer ended
    # exactly at the end of the file without touching EOF
    assert nb in (len(want), len(want) + 1)
    for b, (s, e) in enumerate(want):
        buf = oracle_lib.filter_species(synth.subset(ev, s, e), mon)
        assert nev[b] == buf.n_events
        assert npart[b] == buf.n_particles
        if mixed is None:
            assert mnev[b] == buf.n_events and mpart[b] == buf.n_particles
    if mixed is not None:
        mwant = oracle_lib.buffer_ranges(mixed.multiplicities(), size)
        for b, (s, e) in enumerate(mwant[:len(want)]):
            mb = oracle_lib.filter_species(synth.subset(mixed, s, e), mon)
            assert mnev[b] == mb.n_events and mpart[b] == mb.n_particles


@pytest.mark.parametrize("name", CASES)
def test_writer_reproduces_reference_files(host, name, tmp_path):
    """Oracle histograms written by the drop-in writer == reference files."""
    _check_writer(host, name, tmp_path, oracle_lib.GOLDEN)


def _check_writer(host, name, tmp_path, root):
    orc = oracle_lib.run_golden_case_through_oracle(name, str(tmp_path), root)
    h = orc.hist()
    out = tmp_path / "w"
    out.mkdir()
    p = orc.p
    hp = engine.HbtParams(qnpts=p["qnpts"], q_min=p["q_min"], q_max=p["q_max"], n_KT=p["n_KT"],
                          KT_min=p["KT_min"], KT_max=p["KT_max"], n_Kphi=p["n_Kphi"],
                          azimuthal_flag=p["azimuthal_flag"],
                          invariant_radius_flag=p["invariant_radius_flag"])
    prm, _, _ = oracle_lib.golden_case(name, root)
    arrs = [np.ascontiguousarray(h[k]) for k in
            ("count", "q_out", "q_side", "q_long", "num", "den",
             "qinv_sum", "qinv_num", "qinv_count", "qinv_den")]
    ctr = [np.ascontiguousarray(h[k]) for k in
           ("ctr_num", "ctr_den", "ctr_num_qinv", "ctr_den_qinv")]
    rc = host.hbt_host_write(ctypes.byref(hp), str(out).encode(), int(prm.get("ecooutput", 0)),
                             *[a.ctypes.data_as(_PD) for a in arrs],
                             *[c.ctypes.data_as(_PU) for c in ctr])
    assert rc == 0
    with tarfile.open(os.path.join(root, name, "outputs.tar.gz")) as tar:
        want = {m.name: tar.extractfile(m).read() for m in tar.getmembers()}
    got = {f: open(os.path.join(out, f), "rb").read() for f in os.listdir(out)}
    assert sorted(got) == sorted(want)
    for f in want:
        parity.same_output_file(got[f], want[f], f)


SWEEP = [("mode10", k) for k in range(24)] + [("oscar", k) for k in range(8)]


def _sweep_case(kind, k):
    import sys
    sys.path.insert(0, os.path.join(oracle_lib.REPO, "tests", "golden"))
    import make_golden
    case = make_golden.random_case(k) if kind == "mode10" else make_golden.random_oscar_case(k)
    return make_golden, case


@pytest.mark.parametrize("kind,k", SWEEP)
def test_reader_buffers_on_random_parameter_sets(host, kind, k, tmp_path):
    """The buffering check on the random cases of make_golden (buffer sizes
    from one event to 400 particles, species filters, real mixed-event
    files)."""
    mg, case = _sweep_case(kind, k)
    root = str(tmp_path / "cases")
    mg.write_case("c", case, root)
    _check_buffers(host, "c", str(tmp_path), root)


@pytest.mark.slow
@pytest.mark.parametrize("kind,k", SWEEP)
def test_writer_on_random_parameter_sets(host, kind, k, tmp_path):
    """Where the reference checkout is on this machine: the writer, fed the
    oracle's histograms of a random case, reproduces the files the
    reference binary writes for it (grid sizes, K_T edges in the file names,
    K_phi and q_inv files)."""
    mg, case = _sweep_case(kind, k)
    ref = oracle_lib.reference_checkout()
    if not ref or not os.path.exists(mg.REF_BIN):
        pytest.skip("no reference checkout or no oracle/_ref binary")
    root = str(tmp_path / "cases")
    import contextlib
    import io
    with contextlib.redirect_stdout(io.StringIO()):
        mg.run_case("c", case, ref, out_root=root)
    _check_writer(host, "c", tmp_path, root)


# ------------------------------------------------------------------ readers

def _bind_digest(L):
    L.hbt_host_digest_buffers.restype = ctypes.c_int
    L.hbt_host_digest_buffers.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32,
                                          ctypes.POINTER(ctypes.c_char_p), ctypes.c_int32,
                                          ctypes.POINTER(ctypes.c_uint64)]


def _digests(L, pfile, res, args, cap=4096):
    _bind_digest(L)
    argv = (ctypes.c_char_p * max(len(args), 1))(*[a.encode() for a in args])
    out = (ctypes.c_uint64 * cap)()
    n = L.hbt_host_digest_buffers(pfile.encode(), res.encode(), len(args), argv, cap, out)
    return n, list(out[:max(n, 0)])


@pytest.mark.parametrize("name", CASES)
def test_block_reader_equals_line_reader_on_golden_inputs(host, name, tmp_path):
    """The parallel block reader gives bit-identical particles, buffer by
    buffer, to the line-by-line reader (the reference's reading rule)."""
    pfile, res = _stage(name, str(tmp_path))
    n0, d0 = _digests(host, pfile, res, ["hbt_fast_reader=0"])
    assert n0 > 0
    for threads in (0, 1, 3):
        n1, d1 = _digests(host, pfile, res, ["hbt_fast_reader=1",
                                             "hbt_reader_threads=%d" % threads])
        assert (n1, d1) == (n0, d0)


def _write_text(path, text, gz):
    if gz:
        import gzip
        with gzip.open(path, "wt", newline="") as f:
            f.write(text)
    else:
        with open(path, "w", newline="") as f:
            f.write(text)


def _mode10_text(rng, mults, fmt="%.17g", eol="\n", final_newline=True, plus=False):
    lines = []
    for m in mults:
        lines.append("%d" % m)
        for _ in range(m):
            v = [211, 0.13957] + list(rng.normal(0, 3, 4)) + [abs(rng.normal(1, 0.3)) + 0.2] + \
                list(rng.normal(0, 0.4, 3))
            tok = ["%d" % v[0]] + [fmt % x for x in v[1:]]
            if plus:
                tok = [("+" + t if not t.startswith("-") and k % 3 == 1 else t)
                       for k, t in enumerate(tok)]
            lines.append(" ".join(tok))
    text = eol.join(lines)
    return text + eol if final_newline else text


@pytest.mark.parametrize("variant", ["plain", "no_final_newline", "crlf", "plus_signs",
                                     "scientific", "empty_events", "exact_fill"])
def test_block_reader_equals_line_reader_on_edge_files(host, variant, tmp_path):
    rng = np.random.default_rng(zlib.crc32(variant.encode()))
    mults = list(rng.integers(0, 40, size=23))
    kw = {}
    size = 100
    if variant == "no_final_newline":
        kw["final_newline"] = False
    elif variant == "crlf":
        kw["eol"] = "\r\n"
    elif variant == "plus_signs":
        kw["plus"] = True
    elif variant == "scientific":
        kw["fmt"] = "%.10E"
    elif variant == "empty_events":
        mults = [0, 0, 5, 0, 17, 0, 0, 3, 0]
    elif variant == "exact_fill":
        mults = [25] * 8   # buffers end exactly at the end of the file
    res = tmp_path / "results"
    res.mkdir()
    _write_text(str(res / "particle_samples.gz"), _mode10_text(rng, mults, **kw), gz=True)
    prm = open(os.path.join(oracle_lib.GOLDEN, "basic", "parameters.dat")).read()
    prm = prm.replace("event_buffer_size = 120", "event_buffer_size = %d" % size)
    pfile = tmp_path / "parameters.dat"
    pfile.write_text(prm)
    n0, d0 = _digests(host, str(pfile), str(res), ["hbt_fast_reader=0"])
    n1, d1 = _digests(host, str(pfile), str(res), ["hbt_fast_reader=1", "hbt_reader_threads=4"])
    assert n0 > 0
    assert (n1, d1) == (n0, d0)
    # the binary sidecar: written on the first pass, replayed on the second
    cache = res / "particle_samples.gz.hbtcache"
    assert not cache.exists()
    n2, d2 = _digests(host, str(pfile), str(res), ["hbt_binary_cache=1"])
    assert cache.exists()
    n3, d3 = _digests(host, str(pfile), str(res), ["hbt_binary_cache=1"])
    assert (n2, d2) == (n0, d0) and (n3, d3) == (n0, d0)
    # a changed source file invalidates the sidecar
    os.utime(res / "particle_samples.gz", ns=(1, 1))
    n4, d4 = _digests(host, str(pfile), str(res), ["hbt_binary_cache=1"])
    assert (n4, d4) == (n0, d0)


def test_block_reader_reads_oscar_and_rejects_malformed_lines(host, tmp_path):
    rng = np.random.default_rng(3)
    ev = synth.generate(7, 30.0, seed=4)
    res = tmp_path / "results"
    res.mkdir()
    synth.write_oscar(str(res / "OSCAR.DAT"), ev)
    prm = open(os.path.join(oracle_lib.GOLDEN, "basic", "parameters.dat")).read()
    prm = prm.replace("read_in_mode = 10", "read_in_mode = 0")
    pfile = tmp_path / "parameters.dat"
    pfile.write_text(prm)
    n0, d0 = _digests(host, str(pfile), str(res), ["hbt_fast_reader=0"])
    n1, d1 = _digests(host, str(pfile), str(res), ["hbt_fast_reader=1"])
    assert n0 > 0 and (n1, d1) == (n0, d0)
    # a particle line with a missing column: both readers fail
    bad = _mode10_text(rng, [3, 4]).splitlines()
    bad[3] = " ".join(bad[3].split()[:-1])
    res2 = tmp_path / "bad"
    res2.mkdir()
    _write_text(str(res2 / "particle_samples.gz"), "\n".join(bad) + "\n", gz=True)
    pfile.write_text(open(os.path.join(oracle_lib.GOLDEN, "basic", "parameters.dat")).read())
    for fast in (0, 1):
        n, _ = _digests(host, str(pfile), str(res2), ["hbt_fast_reader=%d" % fast])
        assert n == -1


def test_writer_formats_special_values_like_printf(host, tmp_path):
    """The in-memory writer's %.8e fields equal printf's for signed zeros,
    infinities, subnormals, huge values and values that round at the 8th
    digit (Python's '%e' formatting is correctly rounded, like glibc's)."""
    n, nkt = 3, 2
    nb = nkt * n ** 3
    specials = [0.0, -0.0, float("inf"), -float("inf"), 5e-324, -2.2250738585072014e-308,
                1.7976931348623157e308, 9.9999999950e5, 1.23456785e-7, 2.5e-1, -1.0 / 3.0,
                6.02214076e23, 1.0, -9.99999999e-100, 123456789.0, 1e-5, 0.1, 7.0]
    rng = np.random.default_rng(9)
    cnt = np.full(nb, 2.0)
    cnt[:3] = [0.0, 1.0, 5.0]
    q = [np.array([specials[(k + j) % len(specials)] for k in range(nb)]) for j in range(3)]
    num = np.array([specials[(k + 7) % len(specials)] for k in range(nb)])
    den = rng.integers(0, 50, nb).astype(float)
    den[5] = 1.0
    zeros = [np.zeros(nkt * n) for _ in range(4)]
    ctr = [np.array([3, 0], np.uint64), np.array([7, 1], np.uint64), np.zeros(nkt, np.uint64),
           np.zeros(nkt, np.uint64)]
    hp = engine.HbtParams(qnpts=n, q_min=-0.1, q_max=0.1, n_KT=nkt, KT_min=0.0, KT_max=1.0,
                          n_Kphi=1, azimuthal_flag=0, invariant_radius_flag=0)
    arrs = [cnt] + q + [num, den] + zeros
    assert host.hbt_host_write(ctypes.byref(hp), str(tmp_path).encode(), 0,
                               *[np.ascontiguousarray(a).ctypes.data_as(_PD) for a in arrs],
                               *[c.ctypes.data_as(_PU) for c in ctr]) == 0
    files = os.listdir(tmp_path)
    assert len(files) == 1
    got = open(os.path.join(tmp_path, files[0])).read().split("\n")[:-1]
    grid = [-0.1 + i * 0.1 for i in range(n)]
    ratio = 3.0 / 7.0
    want = []
    for il in range(n):
        for io in range(n):
            for is_ in range(n):
                at = (io * n + is_) * n + il
                if int(cnt[at]) < 2 or int(den[at]) < 2:
                    v = (grid[io], grid[is_], grid[il], 0.0, float(int(den[at])))
                else:
                    c = int(cnt[at])
                    v = (q[0][at] / c, q[1][at] / c, q[2][at] / c, num[at], ratio * den[at])
                want.append("%18.8e    %.8e    %.8e    %.8e    %.8e" % v)
    assert got == want


def test_host_library_exports_every_declared_symbol(host):
    """libhbt_host.so exports every entry point include/hbt_host.h declares."""
    import re
    text = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                             "include", "hbt_host.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = sorted(set(re.findall(r"\b(hbt_host_[a-z_0-9]+)\s*\(", text)))
    assert "hbt_host_run" in names and "hbt_host_event_plane_angle" in names
    for name in names:
        assert hasattr(host, name), name


def _bind_plan(host):
    host.hbt_host_mixed_plan.restype = ctypes.c_int64
    host.hbt_host_mixed_plan.argtypes = [ctypes.c_int32, ctypes.c_int32,
                                         ctypes.POINTER(ctypes.c_int32),
                                         ctypes.POINTER(ctypes.c_int32), ctypes.c_int32,
                                         ctypes.c_int64, ctypes.POINTER(ctypes.c_int32), _PD]


def host_mixed_plan(host, seed, nev, mixed_nev, n_partners):
    """(partners, angles) the drop-in draws for buffers of nev[b] events and
    pools of mixed_nev[b] events."""
    _bind_plan(host)
    nev = np.ascontiguousarray(nev, dtype=np.int32)
    mixed_nev = np.ascontiguousarray(mixed_nev, dtype=np.int32)
    nmix = [n_partners if n_partners > 0 else m // 2 + 1 for m in mixed_nev]
    total = int(sum(int(a) * b for a, b in zip(nev, nmix)))
    partners = np.zeros(max(total, 1), dtype=np.int32)
    angles = np.zeros(max(total, 1))
    _pi = ctypes.POINTER(ctypes.c_int32)
    got = host.hbt_host_mixed_plan(seed, nev.size, nev.ctypes.data_as(_pi),
                                   mixed_nev.ctypes.data_as(_pi), n_partners, total,
                                   partners.ctypes.data_as(_pi), angles.ctypes.data_as(_PD))
    assert got == total
    return partners[:total], angles[:total]


@pytest.mark.parametrize("n_partners", [0, 5])
def test_host_mixed_plan_draws_what_the_oracle_draws(host, n_partners):
    """hbt_host_mixed_plan replays the drop-in's partner and angle draws
    (src/HBT_correlation.cpp:197-217, :495-497); the oracle, pinned to the
    reference's files, draws the same, buffer after buffer, including a
    one-event pool (the reference keeps the event as its own partner)."""
    nev = [11, 10, 1, 7]
    mixed_nev = [11, 10, 1, 9]
    partners, angles = host_mixed_plan(host, 17, nev, mixed_nev, n_partners)
    orc = oracle_lib.Oracle(seed=17, number_of_mixed_events=n_partners)
    L = oracle_lib.lib()
    L.orc_mixed_plan.restype = ctypes.c_int32
    L.orc_mixed_plan.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                 ctypes.POINTER(ctypes.c_int32), _PD]
    at = 0
    for ne, mn in zip(nev, mixed_nev):
        nmix = n_partners if n_partners > 0 else mn // 2 + 1
        p = np.zeros(ne * nmix, dtype=np.int32)
        a = np.zeros(ne * nmix)
        assert L.orc_mixed_plan(orc._h, ne, mn, p.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                a.ctypes.data_as(_PD)) == nmix
        assert np.array_equal(partners[at:at + p.size], p)
        assert np.array_equal(angles[at:at + a.size], a)
        at += p.size
    assert at == partners.size
    # a partner is never the event itself unless the pool has one event
    assert partners[sum(n * (n_partners or m // 2 + 1) for n, m in zip(nev[:2], mixed_nev[:2]))] == 0


def test_host_mixed_plan_rejects_bad_arguments(host):
    _bind_plan(host)
    _pi = ctypes.POINTER(ctypes.c_int32)
    nev = (ctypes.c_int32 * 1)(3)
    empty = (ctypes.c_int32 * 1)(0)
    out = (ctypes.c_int32 * 8)()
    ang = (ctypes.c_double * 8)()
    # an empty pool for a non-empty buffer, a too small cap, negative counts
    assert host.hbt_host_mixed_plan(1, 1, nev, empty, 2, 8, out, ang) == -1
    assert host.hbt_host_mixed_plan(1, 1, nev, nev, 5, 8, out, ang) == -1
    assert host.hbt_host_mixed_plan(1, -1, nev, nev, 2, 8, out, ang) == -1
    assert host.hbt_host_mixed_plan(1, 0, None, None, 2, 0, None, None) == 0


@pytest.mark.parametrize("fast", [1, 0])
def test_readers_reject_a_truncated_gzip_file(host, fast, tmp_path):
    """A particle_samples.gz cut short anywhere - inside the data, or only
    its 8-byte trailer - is an error for both readers (the line reader and
    the block reader), reported as -1 instead of buffers read from a partial
    stream; the intact file reads as before.  (The reference reads what
    inflates and takes the early end for the end of the file.)"""
    src = os.path.join(oracle_lib.GOLDEN, "basic")
    data = open(os.path.join(src, "particle_samples.gz"), "rb").read()
    res = tmp_path / "results"
    res.mkdir()
    host.hbt_host_digest_buffers.restype = ctypes.c_int
    host.hbt_host_digest_buffers.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32,
                                             ctypes.POINTER(ctypes.c_char_p), ctypes.c_int32,
                                             ctypes.POINTER(ctypes.c_uint64)]
    args = (ctypes.c_char_p * 1)(b"hbt_fast_reader=%d" % fast)
    pfile = os.path.join(src, "parameters.dat").encode()
    for cut in (len(data), len(data) - 4, len(data) - 8, len(data) - 20, len(data) // 2, 10):
        (res / "particle_samples.gz").write_bytes(data[:cut])
        dig = (ctypes.c_uint64 * 256)()
        nb = host.hbt_host_digest_buffers(pfile, str(res).encode(), 1, args, 256, dig)
        if cut == len(data):
            assert nb > 0
        else:
            assert nb == -1, cut


@pytest.mark.parametrize("kind,k", SWEEP)
def test_block_reader_equals_line_reader_on_random_parameter_sets(host, kind, k, tmp_path):
    """The block reader against the line reader on the random cases' inputs
    and buffer sizes (both readers, species filters, real mixed-event
    files): bit-identical particles, buffer by buffer."""
    mg, case = _sweep_case(kind, k)
    root = str(tmp_path / "cases")
    mg.write_case("c", case, root)
    pfile, res = _stage("c", str(tmp_path), root)
    n0, d0 = _digests(host, pfile, res, ["hbt_fast_reader=0"])
    assert n0 > 0
    n1, d1 = _digests(host, pfile, res, ["hbt_fast_reader=1", "hbt_reader_threads=3"])
    assert (n1, d1) == (n0, d0)
