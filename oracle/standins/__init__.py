"""Stand-ins for the reference's third-party imports that neither host has (h5py,
psutil on Arm, asciiplotlib, plotly), so that the reference's own command-line front end
(gravitation benchmark / worker / analyze) can run unchanged with the gb1 kernel
(oracle/frontend.py puts this directory on the front end's PYTHONPATH).  Each provides
only what the reference's modules touch at import or on the code paths used; this file
itself is not imported by them."""
