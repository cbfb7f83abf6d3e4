"""Stand-in for plotly.offline.plot (see the package docstring)."""


def plot(*args, **kwargs):
    raise RuntimeError('plotly is not installed; the plot command is not available')
