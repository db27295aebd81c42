"""Sub-box temperature log (data_write, src/heatflow/mod_output.f90:57-66, :92-113, :186-199).

After step `itime` the reference logs `real((itime-1)*time_step)` and the sub-box
`start_ix:end_ix, start_iy:end_iy, start_iz:end_iz` of Temp_pp -- the field before the step's
solution, i.e. the temperature at time (itime-1)*dt -- once when it opens the log at itime = 1
(:79-98), and again whenever _WriteToTxt is set and mod(itime, write_every) = 0 (:104-113), into
./outputs/output_<RunName>_NN with NN the first unused two-digit index (last_log, :199-213).  The
two rules are independent, so with write_every = 1 step 1 is logged twice.  Here the steps run on
the GPU in chunks between records; after each chunk the sub-box is gathered on the device and
copied to pinned host memory on a separate stream (hf_subbox_async), and a writer thread formats
the record while the next chunk runs.

Records are written one per line: the time in single precision (the reference converts it with
real()), then the box values x fastest, as list-directed-style scientific numbers.
"""
from __future__ import annotations

import os
import queue
import threading
from typing import Optional, Sequence

import numpy as np


def next_log_name(outdir: str, run_name: str) -> str:
    """First `output_<RunName>_NN` (NN two digits, from 00) that does not exist in outdir."""
    i = 0
    while True:
        name = os.path.join(outdir, f"output_{run_name.strip()}_{i:02d}")
        if not os.path.exists(name):
            return name
        i += 1


def records_after(itime: int, write_every: int, write_to_txt: bool = True,
                  test_run: bool = False) -> int:
    """How many records data_write appends after step `itime` (mod_output.f90:79-113)."""
    if test_run:
        return 0
    n = 1 if itime == 1 else 0
    if write_to_txt and write_every > 0 and itime % write_every == 0:
        n += 1
    return n


def format_record(time: float, values: np.ndarray) -> str:
    t = float(np.float32(time))
    return " " + " ".join([f"{t:15.8E}"] + [f"{v:24.16E}" for v in np.ravel(values)]) + "\n"


def parse_records(text: str):
    """[(time, values)] from a log written by `format_record`."""
    out = []
    for line in text.splitlines():
        parts = line.split()
        if parts:
            out.append((float(parts[0]), np.array([float(p) for p in parts[1:]])))
    return out


def _host_buffer(n: int) -> np.ndarray:
    try:   # pinned memory lets the copy engine run while the next steps compute
        import torch
        if torch.cuda.is_available():
            return torch.empty(n, dtype=torch.float64).pin_memory().numpy()
    except Exception:
        pass
    return np.empty(n)


class SubboxLog:
    """Run steps and log a sub-box the reference's way, overlapping the copies with stepping.

    hf: a HeatFlow context; lo/hi: 0-based inclusive (x, y, z) corners of the box (the
    reference's start_i-1 .. end_i-1); write_every, write_to_txt, test_run: the reference's
    write_every, _WriteToTxt and _TestRun (records_after).
    """

    def __init__(self, hf, lo: Sequence[int], hi: Sequence[int], write_every: int, path: str,
                 time_step: float, instance: int = 0, write_to_txt: bool = True,
                 test_run: bool = False):
        self.hf, self.lo, self.hi = hf, tuple(lo), tuple(hi)
        self.write_every, self.path, self.dt, self.instance = int(write_every), path, time_step, instance
        self.write_to_txt, self.test_run = bool(write_to_txt), bool(test_run)
        self.n = int(np.prod([h - l + 1 for l, h in zip(self.lo, self.hi)]))
        self._bufs = [_host_buffer(self.n) for _ in range(4)]
        self._q: queue.Queue = queue.Queue(maxsize=3)
        self._err: Optional[BaseException] = None

    def _writer(self, f):
        while True:
            item = self._q.get()
            if item is None:
                return
            ticket, itime, buf, copies = item
            try:
                self.hf.subbox_wait(ticket)
                f.write(format_record((itime - 1) * self.dt, buf) * copies)
            except BaseException as e:       # surfaced by run()
                self._err = e

    def run(self, itime0: int, nsteps: int) -> dict:
        """Steps itime0 .. itime0 + nsteps - 1, logging as records_after says."""
        copies = {k: records_after(k, self.write_every, self.write_to_txt, self.test_run)
                  for k in range(itime0, itime0 + nsteps)}
        marks = [k for k, c in copies.items() if c > 0]
        stats = {"steps": 0, "records": 0}
        with open(self.path, "a") as f:
            th = threading.Thread(target=self._writer, args=(f,), daemon=True)
            th.start()
            try:
                k, slot = itime0, 0
                last = itime0 + nsteps - 1          # steps after the last record run too
                for m in marks + ([] if copies.get(last) else [last]):
                    if m >= k:
                        st = self.hf.run(k, m - k + 1)
                        stats["steps"] += st["steps"]
                        k = m + 1
                    if m in marks:
                        buf = self._bufs[slot % len(self._bufs)]
                        ticket, _ = self.hf.subbox_async(self.lo, self.hi, which=1, out=buf,
                                                         instance=self.instance)
                        self._q.put((ticket, m, buf, copies[m]))   # blocks 3 records behind
                        slot += 1
                        stats["records"] += copies[m]
            finally:
                self._q.put(None)
                th.join()
        if self._err is not None:
            raise self._err
        return stats
