"""The bench's clock sampler (bench.Clocks) on the host, against a stand-in
nvidia-smi that prints the queried CSV fields: it is running before the timed
region starts, it takes a sample after the region ends, and it reports the
median SM clock, the maximum and the throttle reasons that were active.
No GPU needed."""
import importlib
import os
import stat
import sys
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture()
def fake_smi(tmp_path, monkeypatch):
    def make(lines):
        script = tmp_path / 'nvidia-smi'
        body = '\n'.join('echo "%s"; sleep 0.02' % ln for ln in lines)
        script.write_text('#!/bin/bash\nwhile true; do\n%s\ndone\n' % body)
        script.chmod(script.stat().st_mode | stat.S_IEXEC)
        monkeypatch.setenv('PATH', str(tmp_path) + os.pathsep + os.environ.get('PATH', ''))
    return make


@pytest.fixture()
def bench(monkeypatch):
    monkeypatch.syspath_prepend(ROOT)
    monkeypatch.setattr(sys, 'argv', ['bench.py'])
    return importlib.import_module('bench')


def test_sampler_brackets_the_region(bench, fake_smi):
    fake_smi(['0, 2070, 2070, 700.0, 0x0, Not Active, Not Active, Not Active, Not Active',
              '0, 1980, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active'])
    c = bench.Clocks(0)
    assert c._lines() >= 1  # sampling was running before the region
    time.sleep(0.01)        # a region far shorter than the sampling period
    r = c.stop()
    assert r['samples'] >= 2
    assert r['sm_max_mhz'] == 2070.0
    assert r['sm_mhz'] in (1980.0, 2025.0, 2070.0)
    assert r['reasons'] == ['sw_power_cap']  # from the second line, sampled after the region


def test_sampler_reports_slowdown_reasons(bench, fake_smi):
    fake_smi(['0, 1500, 2070, 1400.0, 0x8, Active, Not Active, Active, Not Active'])
    r = bench.Clocks(0).stop()
    assert r['reasons'] == ['hw_slowdown', 'sw_thermal_slowdown']
    assert r['sm_mhz'] == 1500.0


def test_sampler_without_nvidia_smi(bench, tmp_path, monkeypatch):
    monkeypatch.setenv('PATH', str(tmp_path))  # no nvidia-smi here
    t0 = time.time()
    assert bench.Clocks(0).stop() is None
    assert time.time() - t0 < 2.0
