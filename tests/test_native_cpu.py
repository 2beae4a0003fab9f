"""The native library on the CPU: exports, host-side parsing/generation, argument errors.

No kernel runs here; everything below is host code of libgputucker_gb300.so
(the GPU paths are in the tests marked gpu).
"""

import ctypes as C
import glob
import os
import re
import subprocess

import numpy as np
import pytest

import gputucker_gb300 as gtk
from gputucker_gb300 import _native as nat
from oracle_util import ROOT, ora_parse

HEADER = os.path.join(ROOT, "include", "gputucker_gb300.h")
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "*.npz")))


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gtk_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_function(native):
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(native, n)]
    assert not missing, missing
    # and the Python binding declares a signature for each
    assert set(names) <= set(nat.SIGNATURES), set(names) - set(nat.SIGNATURES)


def test_version(native):
    assert native.gtk_version() == 1


PARSE_TEXTS = [
    b"1\t2\t3\t0.5\n2 3 4 0.25\n",
    b"1\t2\t3\t0.5\n4\t4\t4\t1.5\ntrailing text without newline",
    b"1\t1\t1\n2\t2\t2\t0.75\n3\t3\t3\n5\t1\t2\n",
    b"1\t2\t3\t0.5\r\n2\t3\t4\t0.25\r\n",
    b"  1 \t 2\t3   7e-1\n",
    b"7\t8\t9\t1e-3 extra tokens ignored\n",
    b"",
    b"no newline at all",
]


def _value_tokens(rng, n):
    """Value tokens in the forms tensor files hold, and the edge cases of the
    parser's exact decimal fast path (digit counts around 19, exponents around
    +-22, signed zeros, forms it leaves to strtod)."""
    toks = []
    x = rng.random(n)
    toks += [f"{v:.9g}" for v in x.astype(np.float32)]
    toks += [f"{v:.17g}" for v in x[: n // 4]]
    toks += [f"{v:.6e}" for v in rng.lognormal(0, 8, n // 4)]
    toks += [f"{v:.15g}" for v in rng.normal(0, 1e3, n // 4)]
    toks += [str(int(v)) for v in rng.integers(0, 10 ** 12, n // 8)]
    toks += ["0", "-0", "+0.0", "0.000", "1", "-1", "5.", ".5", "-.25", "+7", "1e5", "1E-5", "2.5e+3",
             "0.1e2", "123456789012345678", "1234567890123456789", "12345678901234567890",
             "9007199254740993", "9007199254740992", "0.30000000000000004", "1e22", "1e23", "1e-22",
             "1e-23", "4.9e-324", "1.7976931348623157e308", "1e400", "1e-400", "0x1p-3", "inf", "-nan",
             "1.5abc", "3.14159265358979323846264338327950288", "000000000000000000000001.5",
             "0.0000000000000000000000000001234", "7e0", "1e+0022", "123.456e-10"]
    return toks


@pytest.mark.parametrize("dtype", [0, 1])
def test_parser_values_match_correct_rounding(native, dtype):
    """Every value token reads as strtod reads it (a correctly rounded double,
    then narrowed to value_t): against Python's float(), also correctly rounded,
    for the tokens the fast path takes and those it leaves to strtod."""
    rng = np.random.default_rng(11)
    toks = _value_tokens(rng, 4000)
    text = "".join(f"{i % 7 + 1}\t{i % 5 + 1}\t{i % 3 + 1}\t{t}\n" for i, t in enumerate(toks)).encode()
    coo = gtk.parse_buffer(text, 3, dtype, rand_seed=1)
    _, gv = coo.arrays()
    want = []
    for t in toks:
        m = re.match(r"[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?", t)
        if t.lower().lstrip("+-").startswith(("inf", "nan")) or t.startswith("0x"):
            want.append(float.fromhex(t) if t.startswith("0x") else float(t))
        else:
            want.append(float(m.group(0)))
    want = np.array(want, dtype=np.float64)
    if dtype == 0:
        with np.errstate(over="ignore"):  # 1e400 and the like narrow to inf, as in C
            want = want.astype(np.float32)
    got = gv
    same = (got == want) | (np.isnan(got) & np.isnan(want))
    assert same.all(), [(toks[i], got[i], want[i]) for i in np.flatnonzero(~same)[:10]]
    # signs of zeros too
    assert np.array_equal(np.signbit(got), np.signbit(want))


@pytest.mark.parametrize("text", PARSE_TEXTS)
@pytest.mark.parametrize("dtype", [0, 1])
def test_parser_matches_oracle(native, text, dtype):
    rc, idx, vals, dims, draws = ora_parse(text, 3, dtype, seed=1)
    assert rc == 0
    coo = gtk.parse_buffer(text, 3, dtype, rand_seed=1)
    gi, gv = coo.arrays()
    assert coo.nnz == len(vals)
    if coo.nnz:
        assert coo.dims == dims
    assert coo.rand_draws == draws
    for n in range(3):
        np.testing.assert_array_equal(gi[n], idx[n])
    np.testing.assert_array_equal(gv, vals)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_parser_mixed_line_forms_match_oracle(native, seed):
    """Lines in the common form (the parser's one-pass path) mixed with every
    other form it hands to its general path -- blanks before, between and after
    tokens, extra columns, signed and zero-padded indices, exponents, CRLF,
    missing values -- give the oracle's indices, values, dims and draws."""
    rng = np.random.default_rng(seed)
    lines = []
    for i in range(3000):
        a, b, c = (int(x) for x in rng.integers(1, 50, 3))
        v = f"{rng.random():.9g}"
        form = int(rng.integers(0, 10))
        if form < 4:
            lines.append(f"{a}\t{b}\t{c}\t{v}\n")
        elif form == 4:
            lines.append(f"  {a} \t {b}\t{c}   {v}  \n")
        elif form == 5:
            lines.append(f"{a}\t{b}\t{c}\t{v}\textra\t9\n")
        elif form == 6:
            lines.append(f"+{a}\t00{b}\t{c}\t{v}e0\n")
        elif form == 7:
            lines.append(f"{a}\t{b}\t{c}\t{v}\r\n")
        elif form == 8:
            lines.append(f"{a}\t{b}\t{c}\n")  # value drawn from rand()
        else:
            lines.append(f"{a} {b} {c} -{v}E-2\n")
    text = "".join(lines).encode()
    for dtype in (0, 1):
        rc, idx, vals, dims, draws = ora_parse(text, 3, dtype, seed=seed)
        assert rc == 0
        coo = gtk.parse_buffer(text, 3, dtype, rand_seed=seed)
        gi, gv = coo.arrays()
        assert coo.dims == dims and coo.rand_draws == draws
        for n in range(3):
            np.testing.assert_array_equal(gi[n], idx[n])
        np.testing.assert_array_equal(gv, vals)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_parser_matches_reference_golden(native, path):
    g = np.load(path)
    N = len(g["dims"])
    coo = gtk.parse_from_file(path[:-4] + ".tns", N, int(g["dtype"]), rand_seed=1)
    idx, vals = coo.arrays()
    assert coo.dims == [int(x) for x in g["dims"]]
    assert coo.rand_draws == int(g["skip"])
    for n in range(N):
        np.testing.assert_array_equal(idx[n], g[f"parsed_idx{n}"])
    np.testing.assert_array_equal(vals, g["parsed_vals"])


@pytest.mark.parametrize("text,code", [
    (b"1\t0\t3\t0.5\n", nat.GTK_ERR_PARSE),         # 0 is not a 1-based index
    (b"1\t2\n", nat.GTK_ERR_PARSE),                 # fewer indices than the order
    (b"1\t2\t3\t0.5\n\n", nat.GTK_ERR_PARSE),       # empty line
    (b"1\t2\t3\tabc\n", nat.GTK_ERR_PARSE),         # value that is not a number
    (b"# comment\n1\t2\t3\t0.5\n", nat.GTK_ERR_PARSE),  # the format has no comments
    (b"1\t4294967296\t3\t0.5\n", nat.GTK_ERR_PARSE),  # narrows to index 0 as a uint32
])
def test_parser_errors(native, text, code):
    with pytest.raises(gtk.GTKError) as e:
        gtk.parse_buffer(text, 3, "f64")
    assert e.value.code == code


def test_parse_missing_file(native):
    with pytest.raises(gtk.GTKError) as e:
        gtk.parse_from_file("/nonexistent/x.tns", 3)
    assert e.value.code == nat.GTK_ERR_IO


@pytest.mark.parametrize("order", [0, 9])
def test_parse_bad_order(native, order):
    with pytest.raises(gtk.GTKError) as e:
        gtk.parse_buffer(b"1 1 1 1\n", order)
    assert e.value.code == nat.GTK_ERR_ARG


def test_parser_large_multithreaded_matches_oracle(native, tmp_path):
    coo = gtk.generate(3, [5000, 6000, 7000], 300_000, "zipf", 1.2, "uniform", "f64", seed=3)
    p = tmp_path / "big.tns"
    coo.write_text(str(p))
    data = p.read_bytes()
    rc, idx, vals, dims, _ = ora_parse(data, 3, 1)
    assert rc == 0
    back = gtk.parse_from_file(str(p), 3, "f64")
    bi, bv = back.arrays()
    gi, gv = coo.arrays()
    for n in range(3):
        np.testing.assert_array_equal(bi[n], idx[n])
        np.testing.assert_array_equal(bi[n], gi[n])
    np.testing.assert_array_equal(bv, vals)
    np.testing.assert_array_equal(bv, gv)  # %.17g round-trips doubles
    assert back.dims == dims == coo.dims


def test_f32_text_roundtrip(native, tmp_path):
    coo = gtk.generate(4, [300] * 4, 20_000, "uniform", 0, "uniform", "f32", seed=1)
    p = tmp_path / "f.tns"
    coo.write_text(str(p))
    back = gtk.parse_from_file(str(p), 4, "f32")
    np.testing.assert_array_equal(back.arrays()[1], coo.arrays()[1])


def test_generator_deterministic_and_distinct(native):
    a = gtk.generate(4, [1000] * 4, 50_000, "zipf", 1.1, "uniform", "f32", seed=5)
    b = gtk.generate(4, [1000] * 4, 50_000, "zipf", 1.1, "uniform", "f32", seed=5)
    c = gtk.generate(4, [1000] * 4, 50_000, "zipf", 1.1, "uniform", "f32", seed=6)
    ai, av = a.arrays()
    bi, bv = b.arrays()
    ci, _ = c.arrays()
    for n in range(4):
        np.testing.assert_array_equal(ai[n], bi[n])
    np.testing.assert_array_equal(av, bv)
    assert any((ai[n] != ci[n]).any() for n in range(4))
    keys = np.stack(ai, 1)
    assert len(np.unique(keys, axis=0)) == len(keys)
    # power-law slices: the heaviest slice holds far more than the mean
    counts = np.bincount(ai[0])
    assert counts.max() > 20 * counts.mean()
    assert av.min() >= 0 and av.max() < 1


def test_generator_lognormal_scaled(native):
    a = gtk.generate(3, [2000] * 3, 20_000, "zipf", 1.05, "lognormal", "f32", seed=2)
    v = a.arrays()[1]
    assert v.max() == pytest.approx(1.0) and v.min() > 0


def test_generator_planted(native):
    a = gtk.generate_planted(3, [200] * 3, 5000, 4, 0.01, "f32", seed=1)
    v = a.arrays()[1]
    assert a.nnz == 5000 and v.mean() > 1.0  # sum of 64 positive products


@pytest.mark.parametrize("P,code", [([6, 1, 1], nat.GTK_ERR_PARTITION), ([0, 1, 1], nat.GTK_ERR_ARG)])
def test_create_blocks_rejects_bad_partition(native, P, code):
    coo = gtk.coo_from_arrays([np.array([0, 9], np.uint32)] * 3, np.array([1.0, 2.0]), dims=[10, 10, 10])
    with pytest.raises(gtk.GTKError) as e:
        gtk.create_tensor_blocks(coo, P, 4)
    assert e.value.code == code


@pytest.mark.parametrize("rank", [0, 65])
def test_create_blocks_rejects_rank(native, rank):
    coo = gtk.coo_from_arrays([np.array([0, 1], np.uint32)] * 3, np.array([1.0, 2.0]))
    with pytest.raises(gtk.GTKError) as e:
        gtk.create_tensor_blocks(coo, [1, 1, 1], rank)
    assert e.value.code == nat.GTK_ERR_ARG


def test_coo_from_arrays_bounds(native):
    with pytest.raises(gtk.GTKError) as e:
        gtk.coo_from_arrays([np.array([0, 10], np.uint32)] * 2, np.array([1.0, 2.0]), dims=[10, 10])
    assert e.value.code == nat.GTK_ERR_ARG


def test_cli_usage(native):
    from gputucker_gb300 import build
    cli = build.CLI
    assert os.path.exists(cli)
    r = subprocess.run([cli, "-h"], capture_output=True, text=True)
    assert r.returncode == 0 and "--input" in r.stdout
    r = subprocess.run([cli, "-o", "3"], capture_output=True, text=True)
    assert r.returncode == 2 and "Input file must be specified" in r.stdout
    r = subprocess.run([cli, "-i", "/nonexistent", "-o", "3"], capture_output=True, text=True)
    assert r.returncode == 2


# ---- partition planner (Optimizer::FindPartitionParms, optimizer.tpp:71-89)
def _plan(native, dims, nnz, rank, dtype, gpus, mem):
    plan = nat.Plan()
    d = np.ascontiguousarray(dims, dtype=np.uint32)
    rc = native.gtk_plan_partition(len(dims), d.ctypes.data_as(nat.U32P), nnz, rank, dtype, gpus, mem,
                                   C.byref(plan))
    N = len(dims)
    return rc, list(plan.partition_dims[:N]), list(plan.block_dims[:N]), plan


def test_planner_matches_reference_golden(native):
    """Every case of planner_cases.json (produced by the reference's own optimizer)."""
    import json
    cases = json.load(open(os.path.join(ROOT, "tests", "golden", "planner_cases.json")))
    assert len(cases) >= 15
    for c in cases:
        rc, P, bd, plan = _plan(native, c["dims"], c["nnz"], c["rank"], c["dtype"], c["gpus"], c["mem"])
        if c["status"] != 0:  # the reference threw
            assert rc == nat.GTK_ERR_PARTITION, c
            continue
        assert rc == 0, (c, native.gtk_last_error())
        assert P == c["P"] and bd == c["block_dims"], c
        assert plan.block_count == c["block_count"] and plan.dimension_based == c["dimension_based"], c
        assert plan.streams == c["streams"] and plan.avail_nnz_per_task == c["avail_nnz_per_task"], c


def test_planner_matches_reference_random(native):
    """Random shapes and memory sizes against the reference compiled in place (when built)."""
    from oracle_util import ref_available, ref_plan
    if not ref_available():
        pytest.skip("oracle/_ref not built")
    rng = np.random.default_rng(5)
    for _ in range(300):
        N = int(rng.integers(1, 9))
        dims = [int(x) for x in np.exp(rng.uniform(0, np.log(3e6), N)).astype(np.int64) + 1]
        nnz = int(np.exp(rng.uniform(0, np.log(2e9))))
        J = int(rng.integers(1, 33))
        dt = int(rng.integers(0, 2))
        gpus = int(rng.integers(1, 9))
        mem = int(np.exp(rng.uniform(np.log(1e4), np.log(3e11))))
        st, P, bd, nblk, dim_based, streams, avail = ref_plan(dims, nnz, J, dt, gpus, mem)
        rc, P2, bd2, plan = _plan(native, dims, nnz, J, dt, gpus, mem)
        if st != 0:
            assert rc == nat.GTK_ERR_PARTITION
            continue
        assert rc == 0 and P2 == P and bd2 == bd, (dims, nnz, J, dt, gpus, mem, P, P2)
        assert (plan.block_count, plan.dimension_based, plan.streams, plan.avail_nnz_per_task) == \
            (nblk, dim_based, streams, avail)


def test_planner_rejects_bad_arguments(native):
    assert _plan(native, [10, 0], 5, 4, 0, 1, 1 << 30)[0] == nat.GTK_ERR_ARG
    assert _plan(native, [10, 10], 5, 0, 0, 1, 1 << 30)[0] == nat.GTK_ERR_ARG
    assert _plan(native, [10, 10], 5, 4, 7, 1, 1 << 30)[0] == nat.GTK_ERR_ARG
    assert _plan(native, [10, 10], 5, 4, 0, 0, 1 << 30)[0] == nat.GTK_ERR_ARG


def test_checkpoint_info_rejects_garbage(native, tmp_path):
    p = tmp_path / "x.ckpt"
    p.write_bytes(b"definitely not a checkpoint file")
    assert native.gtk_checkpoint_info(str(p).encode(), None, None, None, None, None, None) == nat.GTK_ERR_PARSE
    assert native.gtk_checkpoint_info(str(tmp_path / "missing").encode(), None, None, None, None, None,
                                      None) == nat.GTK_ERR_IO


@pytest.mark.parametrize("seed,skip,n", [(1, 0, 1000), (7, 123, 300_000), (2**31 + 5, 1_000_007, 200_000)])
def test_random_sequence_jump_ahead(seed, skip, n):
    """gtk_random_sequence (the draws gtk_init_random places) splits the draws over
    host threads, each jumping ahead in glibc's additive recurrence; the values
    must equal frand(0, 1) = rand() / (2^31 - 1) of the C library's own rand()
    stream, draw for draw, whatever the chunk boundaries."""
    libc = C.CDLL("libc.so.6")
    libc.srand.argtypes = [C.c_uint]
    libc.srand(seed & 0xFFFFFFFF)
    for _ in range(skip):
        libc.rand()
    want = np.array([libc.rand() for _ in range(n)], np.float64) / 2147483647.0
    got = np.empty(n, np.float64)
    nat.call("gtk_random_sequence", seed & 0xFFFFFFFF, skip, n, got.ctypes.data)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("skip", [10**9 + 3, 2**40 + 12345, 10**12 + 7])
def test_random_sequence_large_jumps_compose(native, skip):
    """Jumps far beyond what stepping can check: the draws after skip + 5000 are the
    draws after skip, 5000 on (x^(a+b) = x^a x^b mod the recurrence's polynomial),
    and differ from the unskipped stream."""
    a = np.empty(6000, np.float64)
    b = np.empty(1000, np.float64)
    nat.call("gtk_random_sequence", 1, skip, 6000, a.ctypes.data)
    nat.call("gtk_random_sequence", 1, skip + 5000, 1000, b.ctypes.data)
    np.testing.assert_array_equal(b, a[5000:])
    c = np.empty(1000, np.float64)
    nat.call("gtk_random_sequence", 1, 0, 1000, c.ctypes.data)
    assert not np.array_equal(a[:1000], c)
    assert np.all((a >= 0) & (a <= 1))
