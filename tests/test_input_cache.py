"""Binary input cache of the parsed model directory (RLGPU_INPUT_CACHE): the cached load
equals the text parse; the key is the size and modification time of every input file the
parse opened or probed; a damaged or missing cache falls back to the text. Host only."""
import os

import pytest

from radlite_gb300 import synth


@pytest.fixture
def model(tmp_path):
    return synth.write_model(synth.config_by_name("tiny_band"), str(tmp_path / "m"))


@pytest.fixture
def cache_env(tmp_path, monkeypatch):
    d = tmp_path / "cache"
    d.mkdir()
    monkeypatch.setenv("RLGPU_INPUT_CACHE", str(d))
    return d


def load(gpu_lib, d):
    m = gpu_lib.load_dir_host(d)
    c = m.checksum()
    m.free()
    return c


def test_cached_load_equals_text(gpu_lib, model, cache_env, monkeypatch):
    monkeypatch.delenv("RLGPU_INPUT_CACHE")
    text = load(gpu_lib, model)
    monkeypatch.setenv("RLGPU_INPUT_CACHE", str(cache_env))
    assert load(gpu_lib, model) == text          # parses and writes the cache
    files = os.listdir(cache_env)
    assert len(files) == 1 and files[0].endswith(".rlin")
    assert load(gpu_lib, model) == text          # reads the cache


def test_key_is_size_and_mtime(gpu_lib, model, cache_env):
    first = load(gpu_lib, model)
    p = os.path.join(model, "velocity.inp")
    st = os.stat(p)
    txt = open(p).read()
    # same size, same time stamp, other content: the cache still answers
    lines = txt.rstrip("\n").split("\n")
    last = lines[-1]
    k = len(last) - 1 - last[::-1].index("e") - 1        # the mantissa's last digit of the final value
    lines[-1] = last[:k] + str((int(last[k]) + 1) % 10) + last[k + 1:]
    swapped = "\n".join(lines) + "\n"
    assert len(swapped) == len(txt) and swapped != txt
    open(p, "w").write(swapped)
    os.utime(p, ns=(st.st_atime_ns, st.st_mtime_ns))
    assert load(gpu_lib, model) == first
    # a new time stamp: parsed again, and the result differs
    os.utime(p, ns=(st.st_atime_ns, st.st_mtime_ns + 1_000_000))
    second = load(gpu_lib, model)
    assert second != first


def test_probed_file_invalidates(gpu_lib, model, cache_env, monkeypatch):
    load(gpu_lib, model)
    os.remove(os.path.join(model, "starinfo.inp"))      # probed, not required: R* falls back
    cached = load(gpu_lib, model)
    monkeypatch.delenv("RLGPU_INPUT_CACHE")
    assert cached == load(gpu_lib, model)


def test_damaged_cache_falls_back(gpu_lib, model, cache_env, monkeypatch):
    text = load(gpu_lib, model)
    f = os.path.join(cache_env, os.listdir(cache_env)[0])
    data = open(f, "rb").read()
    open(f, "wb").write(data[: len(data) // 2])
    assert load(gpu_lib, model) == text
    monkeypatch.setenv("RLGPU_INPUT_CACHE", os.path.join(str(cache_env), "missing", "dir"))
    assert load(gpu_lib, model) == text
