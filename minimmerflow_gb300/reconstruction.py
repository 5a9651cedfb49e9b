"""Reference-named entry points of src/reconstruction.cpp."""


def initialize():
    """reconstruction::initialize (reconstruction.cpp:34-36): nothing to set up."""


def computePolynomials(solver):
    """reconstruction::computePolynomials (reconstruction.cpp:47-55) on the uploaded state."""
    solver.compute_polynomials()
