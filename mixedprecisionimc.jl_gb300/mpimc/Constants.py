"""Physical constants of a deck: the reference's ``Constants`` module
(src/constants.jl:6-15).  ``set_constants`` parses PHYS_C, PHYS_A and ALPHA in
the deck precision and publishes them as module globals ``phys_c``,
``phys_a`` and ``alpha``, as the Julia module does."""
import numpy as np

phys_c = None
phys_a = None
alpha = None


def parse_p(precision, value):
    """Julia ``parse(precision, s)``: the value rounded to the deck precision."""
    return precision(float(value))


def set_constants(inputs):
    global phys_c, phys_a, alpha
    precision = inputs.get("PRECISION", np.float64)
    phys_c = parse_p(precision, inputs["PHYS_C"])
    phys_a = parse_p(precision, inputs["PHYS_A"])
    alpha = parse_p(precision, inputs["ALPHA"])
    return phys_c, phys_a, alpha
