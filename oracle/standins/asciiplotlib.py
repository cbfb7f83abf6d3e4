"""Stand-in for asciiplotlib, imported by the reference's cli/benchmark.py for its live
terminal plot (display 'plot'); the front end here runs with display 'log' or 'none',
so the figure only needs to exist."""


class _Figure:
    def plot(self, *args, **kwargs):
        pass

    def show(self):
        pass


def figure(*args, **kwargs):
    return _Figure()
