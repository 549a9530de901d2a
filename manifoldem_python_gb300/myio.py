"""Pickle dictionary I/O with the reference's format (``modules/myio.py:21-51``): one dict per
file, protocol ``pickle.HIGHEST_PROTOCOL``; a file that fails to unpickle reads as None.

``AsyncWriter`` writes the per-PD pickles and their resume markers on worker threads while the
GPU computes the next batch (the pickle write, 24 n N^2 bytes per PD, dominates once the stage
itself is fast).  Each task writes its pickle and only then its marker, so a PD counts as done
only when its pickle is complete, as in the reference (``GetDistancesS2.py:29-35``).
"""
import os
import pickle
import threading
from concurrent.futures import ThreadPoolExecutor


def fin1(filename):
    with open(filename, 'rb') as f:
        try:
            return pickle.load(f)
        except Exception:
            return None


def fout1(filename, key_list, v_list):
    to_save = dict((key_list[i], v_list[i]) for i in range(len(key_list)))
    with open(filename, 'wb') as f:
        pickle.dump(to_save, f, protocol=pickle.HIGHEST_PROTOCOL)


def fout2(filename, d):
    fout1(filename, list(d.keys()), list(d.values()))


class AsyncWriter:
    """Pickle writer threads with a bound on the bytes queued but not yet written."""

    def __init__(self, workers: int = 4, max_pending_bytes: int = 8 << 30):
        self._pool = ThreadPoolExecutor(max_workers=max(1, workers))
        self._futures = []
        self._pending = 0
        self._max = max_pending_bytes
        self._cv = threading.Condition()

    @staticmethod
    def _nbytes(values) -> int:
        return sum(int(getattr(v, 'nbytes', 0)) for v in values)

    def submit(self, filename, key_list, v_list, marker=None) -> None:
        """Queue one pickle (and, after it, the empty marker file); blocks while more than
        max_pending_bytes are queued."""
        nb = self._nbytes(v_list)
        with self._cv:
            while self._pending > 0 and self._pending + nb > self._max:
                self._cv.wait()
            self._pending += nb

        def task():
            try:
                fout1(filename, key_list, v_list)
                if marker is not None:
                    open(marker, 'a').close()
            finally:
                with self._cv:
                    self._pending -= nb
                    self._cv.notify_all()

        self._futures.append(self._pool.submit(task))

    def close(self) -> None:
        """Wait for every queued write; re-raise the first error."""
        try:
            for f in self._futures:
                f.result()
        finally:
            self._futures = []
            self._pool.shutdown(wait=True)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False
