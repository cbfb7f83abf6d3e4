"""Stand-in for plotly, imported at import time by the reference's cli/plot.py (the
plot command, which the front end here does not run)."""
