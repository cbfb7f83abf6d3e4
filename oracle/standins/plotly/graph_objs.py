"""Stand-in for plotly.graph_objs (see the package docstring)."""
