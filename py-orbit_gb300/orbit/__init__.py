"""Package ``orbit``: the PyORBIT Python layer (py/orbit) for the 2.5D
space-charge and TEAPOT hot path, running on liborbit_gb300."""
