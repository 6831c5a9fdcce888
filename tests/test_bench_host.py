"""Host-side pieces of bench.py: the CPU baseline leg (also the reference
arm) builds the hash-grid network from a fixed spec and must not load the
product library; the spec must equal the library's preset."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpu_network_spec_matches_library_preset(nmg):
    sys.path.insert(0, ROOT)
    import bench
    spec = nmg.oracle_net_spec(nmg.config(nmg.PRESET_HASHGRID))
    for k, v in bench.HASHGRID_NET.items():
        assert abs(float(spec[k]) - float(v)) < 1e-6, (k, spec[k], v)
    assert set(spec) == set(bench.HASHGRID_NET)


def test_cpu_baseline_does_not_load_the_product_library():
    code = (
        "import sys, importlib, numpy as np; sys.path.insert(0, %r); import bench\n"
        "synth = importlib.import_module(bench.PKG + '.synth')\n"
        "q = synth.wavefront(8192, seed=1)\n"
        "x, rec = synth.train_batch(synth.TrainField(seed=1), 4096, seed=2, input_mode=1, selection=True)\n"
        "r = bench.cpu_baseline(q, x, rec, seconds=0.1)\n"
        "assert r['value'] > 0 and r['kind'] == 'port'\n"
        "print('LOADED' if any('libnmg.so' in l for l in open('/proc/self/maps')) else 'CLEAN')\n" % ROOT)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip().splitlines()[-1] == "CLEAN"
