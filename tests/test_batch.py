"""Host logic of the batched / served executor (no GPU): memory admission and sizing."""
import threading
import time

import pytest

from pymoresane_gb300.batch import MemoryGate, job_bytes


def test_job_bytes_grow_with_size():
    prev = (0, 0)
    for n in (256, 512, 1024, 2048, 4096):
        b, t = job_bytes(n, 2 * n, max(1, n.bit_length() - 4))
        assert b > prev[0] and t > prev[1]
        prev = (b, t)
    # a 2048^2 job with a 4096^2 PSF and 7 scales needs about a gigabyte of buffers
    b, t = job_bytes(2048, 4096, 7)
    assert 0.5e9 < b < 2e9


def test_gate_blocks_until_release():
    gate = MemoryGate(100)
    gate.acquire(70)
    got = threading.Event()

    def second():
        gate.acquire(50)
        got.set()

    t = threading.Thread(target=second)
    t.start()
    time.sleep(0.1)
    assert not got.is_set()          # 70 + 50 > 100: waits
    gate.release(70)
    assert got.wait(2.0)
    t.join()
    assert gate.used == 50


def test_gate_shrinks_before_waiting():
    gate = MemoryGate(100)
    gate.acquire(90)                  # e.g. cached buffers of another image size
    calls = []

    def shrink():
        calls.append(1)
        return 60                     # the worker gives back its cached buffers
    gate.acquire(40, shrink=shrink, timeout=1.0)
    assert calls == [1] and gate.used == 70


def test_gate_rejects_oversized_and_times_out():
    gate = MemoryGate(100)
    with pytest.raises(MemoryError):
        gate.acquire(101)
    gate.acquire(80)
    with pytest.raises(TimeoutError):
        gate.acquire(30, timeout=0.05)
    assert gate.used == 80
