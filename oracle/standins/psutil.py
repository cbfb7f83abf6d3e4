"""Stand-in for psutil.cpu_count, the one psutil call of the reference's front end
(cli/benchmark.py, cli/worker.py: thread-count choices and the platform record)."""
import os


def cpu_count(logical=True):
    return os.cpu_count() or 1
