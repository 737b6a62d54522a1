"""Host-side checks that need no GPU: the C ABI libraries load and export
every symbol their headers declare, the parameter-set table matches the
oracle, the engine's own DRBG/AES match the reference stream, and the
drop-in size queries answer without a device."""
import ctypes
import os
import re

import pytest

from conftest import ROOT, load_golden

INCLUDE = os.path.join(ROOT, "include")


def _declared(header):
    src = open(os.path.join(INCLUDE, header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cuspx_\w+|crypto_sign\w*|randombytes\w*)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    import cuspx_gb300
    return cuspx_gb300.lib()


def test_engine_exports_every_declared_symbol(lib):
    for h in ("cuspx.h", "cuspx_rng.h", "cuspx_serve.h"):
        names = _declared(h)
        assert names, h
        for name in names:
            assert hasattr(lib, name), "%s declared in %s but not exported" % (name, h)


@pytest.mark.parametrize("setname", ["sha256-128f-simple", "shake256-256f-robust", "sha256-128s-simple"])
def test_dropin_exports_and_sizes(setname):
    import cuspx_gb300
    import spx_oracle
    L = ctypes.CDLL(cuspx_gb300.dropin_path(setname))
    for name in _declared("spx_api.h"):
        assert hasattr(L, name), name
    o = spx_oracle.Oracle(setname)
    for fn, want in (("crypto_sign_bytes", o.p.sig_bytes), ("crypto_sign_publickeybytes", o.p.pk_bytes),
                     ("crypto_sign_secretkeybytes", o.p.sk_bytes), ("crypto_sign_seedbytes", o.p.seed_bytes)):
        f = getattr(L, fn)
        f.restype = ctypes.c_ulonglong
        assert f() == want, fn


def test_set_table_matches_oracle():
    import cuspx_gb300 as c
    import spx_oracle
    assert c.num_sets() == 24
    for sid in range(c.num_sets()):
        name = c.set_name(sid)
        o = spx_oracle.Oracle(name)
        z = c.set_sizes(sid)
        assert (z["pk"], z["sk"], z["sig"], z["seed"], z["n"]) == \
            (o.p.pk_bytes, o.p.sk_bytes, o.p.sig_bytes, o.p.seed_bytes, o.p.n), name
        assert c.set_id(name) == sid
    assert c.set_id("sha256-128f") == c.set_id("sha256-128f-simple")
    with pytest.raises(ValueError):
        c.set_id("sha512-128f")


def test_engine_drbg_matches_reference_stream():
    import cuspx_gb300 as c
    import spx_oracle
    g = load_golden("sha256-128f")
    c.randombytes_init(bytes.fromhex(g["entropy"]))
    assert c.randombytes(48).hex() == g["drbg_first48"]
    assert c.randombytes(48).hex() == g["seed"]
    d = spx_oracle.Drbg(bytes(range(48, 96)))
    c.randombytes_init(bytes(range(48, 96)))
    for n in (0, 1, 15, 16, 17, 100):
        assert c.randombytes(n) == d.bytes(n)


def test_engine_aes_known_answers():
    import cuspx_gb300 as c
    assert c.aes256_ecb(bytes(range(32)), bytes.fromhex("00112233445566778899aabbccddeeff")).hex() == \
        "8ea2b7ca516745bfeafc49904b496089"
    import spx_oracle
    import random
    rng = random.Random(3)
    for _ in range(50):
        k = bytes(rng.randrange(256) for _ in range(32))
        p = bytes(rng.randrange(256) for _ in range(16))
        assert c.aes256_ecb(k, p) == spx_oracle.aes256_ecb(k, p)


def test_engine_aes_matches_libcrypto():
    """The reference DRBG calls OpenSSL's AES-256-ECB (rng.cu:116-136); where the
    system libcrypto is present, compare against it directly."""
    import ctypes.util
    path = ctypes.util.find_library("crypto")
    if not path:
        pytest.skip("libcrypto not present")
    C = ctypes.CDLL(path)
    C.EVP_CIPHER_CTX_new.restype = ctypes.c_void_p
    C.EVP_aes_256_ecb.restype = ctypes.c_void_p
    C.EVP_EncryptInit_ex.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p,
                                     ctypes.c_char_p]
    C.EVP_EncryptUpdate.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int),
                                    ctypes.c_char_p, ctypes.c_int]
    C.EVP_CIPHER_CTX_free.argtypes = [ctypes.c_void_p]
    import cuspx_gb300 as c
    import random
    rng = random.Random(4)
    for _ in range(20):
        k = bytes(rng.randrange(256) for _ in range(32))
        p = bytes(rng.randrange(256) for _ in range(16))
        ctx = C.EVP_CIPHER_CTX_new()
        assert C.EVP_EncryptInit_ex(ctx, C.EVP_aes_256_ecb(), None, k, None) == 1
        out = ctypes.create_string_buffer(32)
        n = ctypes.c_int()
        assert C.EVP_EncryptUpdate(ctx, out, ctypes.byref(n), p, 16) == 1
        C.EVP_CIPHER_CTX_free(ctx)
        assert out.raw[:16] == c.aes256_ecb(k, p)


def test_engine_without_gpu_fails_loudly():
    """No CPU fallback: on a machine without a usable GPU the engine refuses."""
    import cuspx_gb300 as c
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except ImportError:
        has_gpu = os.path.exists("/dev/nvidia0")
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(c.CuspxError):
        c.Engine(0)


def test_ctypes_struct_layouts_match_the_headers(tmp_path):
    """The Python bindings' structures have the size and field offsets the C
    headers give them (compiled with the host C compiler)."""
    import shutil
    import subprocess
    import cuspx_gb300 as c
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    cases = {"cuspx_serve_config": c.ServeConfig, "cuspx_serve_counters": c.ServeCounters,
             "cuspx_loadgen_config": c.LoadgenConfig, "cuspx_loadgen_result": c.LoadgenResult,
             "cuspx_loadgen_sample": c.LoadgenSample, "cuspx_tuning": c.Tuning}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "cuspx_serve.h"', "int main(void) {"]
    for cname, py in cases.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", INCLUDE, str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                        text=True).stdout.splitlines())
    for cname, py in cases.items():
        assert int(got[cname]) == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(got[cname + "." + f]) == getattr(py, f).offset, (cname, f)


def test_tuning_file_round_trip(tmp_path):
    """The autotuner's tab-separated tuning file (read by cuspx_create) keeps
    one line per (GPU, set, op, bucket) and round-trips its mappings."""
    from cuspx_gb300 import autotune
    p = str(tmp_path / "t.tsv")
    k1 = ("NVIDIA GB300", "sha256-128f-simple", "verify", 256)
    k2 = ("NVIDIA GB300", "sha256-128f-simple", "sign", 1024)
    autotune.save_entry(k1, 1.25, {"verify_item_max": 256, "verify_mode": 2}, p)
    autotune.save_entry(k2, 20.5, {"leaf_block": 256}, p)
    autotune.save_entry(k1, 1.0, {"verify_item_max": 0, "verify_mode": 2}, p)   # replaces
    c = autotune.load_cache(p)
    assert c == {k1: (1.0, {"verify_item_max": 0, "verify_mode": 2}), k2: (20.5, {"leaf_block": 256})}
    lines = open(p).read().splitlines()
    assert len(lines) == 2 and all(len(x.split("\t")) == 7 for x in lines)
    # each line carries its bucket's item range: 1024 -> 257..1024, 256 -> 65..256
    assert sorted(tuple(x.split("\t")[3:5]) for x in lines) == [("257", "1024"), ("65", "256")]
    assert [autotune.bucket(n) for n in (1, 2, 4, 5, 64, 65, 4096)] == [1, 4, 4, 16, 64, 256, 4096]
    assert [autotune.bucket_range(b) for b in (1, 4, 64)] == [(1, 1), (2, 4), (17, 64)]


def test_autotune_search_space():
    """The verify search covers the sorted and speculative knobs; the
    speculative size limit is only proposed where the library accepts it
    (<= 64 items), and None entries become the bucket's size."""
    import cuspx_gb300 as c
    from cuspx_gb300 import autotune
    small = autotune.search_space(c.OP_VERIFY, 16)
    assert small["verify_spec_max"] == [0, 16] and small["verify_item_max"] == [0, 16]
    assert 3 in small["verify_mode"] and small["verify_groups"] == [2, 4, 6, 8]
    assert autotune.search_space(c.OP_VERIFY, 1024)["verify_spec_max"] == [0]
    assert autotune.search_space(c.OP_VERIFY, 64)["verify_spec_max"] == [0, 64]
    sign = autotune.search_space(c.OP_SIGN, 1024)
    assert "verify_spec_max" not in sign and sign["chain_mode_max"] == [0, 256]
    assert [autotune.bucket(n) for n in (1, 2, 5, 64, 65, 4096)] == [1, 4, 16, 64, 256, 4096]
