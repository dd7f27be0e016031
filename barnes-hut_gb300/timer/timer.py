"""Named wall-clock phases with a median report (python-bh/timer/timer.py:4-57).

Same interface: ``with Timer.get_handle(name): ...``, ``Timer.print()``,
``Timer.reset()``.  Phase names used by the step loop: grid_creation,
summarization, evaluation, timestep, end-to-end.
"""
import statistics
from timeit import default_timer as _now


class TimerHandle:

    def __init__(self, parent, name, verbose):
        self.name = name
        self.parent = parent
        self.verbose = verbose

    def start(self):
        self.t0 = _now()

    def stop(self):
        elapsed = _now() - self.t0
        self.parent._report_time(self.name, elapsed)
        if self.verbose:
            print(f"stopping {self.name}  {elapsed}")

    def __enter__(self):
        if self.verbose:
            print(f"starting {self.name}")
        self.start()
        return self

    def __exit__(self, exc_type, exc, tb):
        self.stop()


class TimerClass:

    def __init__(self):
        self.times = {}
        self.verbose = True

    def get_handle(self, name):
        return TimerHandle(self, name, self.verbose)

    def _report_time(self, name, elapsed):
        self.times.setdefault(name, []).append(elapsed)

    def medians(self, nwarm=0):
        return {k: statistics.median(v[nwarm:]) for k, v in self.times.items() if v[nwarm:]}

    def print(self, nwarm=0):
        print("*" * 50)
        print(f"{'name':<15}, {'median':<7}")
        for name, med in self.medians(nwarm).items():
            print(f"{name:<15}, {med:.5f}")
        print("*" * 50)

    def reset(self):
        self.times = {}


Timer = TimerClass()
