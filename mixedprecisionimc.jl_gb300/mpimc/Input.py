"""Input deck reader: the reference's ``Input.readInputs`` (src/imc_input.jl:20-129).

Same grammar and the same resulting dictionary:

* ``KEY = value`` lines (the regex ``^\\w+ = ``; text after a second ``=`` is
  dropped, as ``split(line, "=")[2]`` drops it), ``#`` comments, blank lines;
* ``[a, b, c]`` arrays on one line or spread over several lines, stored as a
  list of line fragments with the brackets stripped;
* after reading, ``PRECISION`` becomes a numpy float type (HALF/FLOAT16,
  SINGLE/FLOAT32, DOUBLE/FLOAT64) and every other value containing a comma is
  parsed: MESHNODES / XMESHNODES / YMESHNODES always as float64, other arrays
  in the deck precision; arrays containing ``(`` hold tuples.

The reference evaluates tuple arrays with ``eval(Meta.parse(...))``
(src/imc_input.jl:106), which executes deck text.  Here they are parsed as
literals only (``ast.literal_eval``): same tuples, no code execution.
"""
import ast
import re

import numpy as np

_KEY_RE = re.compile(r"^\w+ = ")
_NODE_KEYS = ("MESHNODES", "XMESHNODES", "YMESHNODES")


def precision_set(params):
    """src/imc_input.jl:113-129: map the PRECISION keyword to a float type."""
    if "PRECISION" in params:
        v = params["PRECISION"]
        if v in ("HALF", "FLOAT16"):
            params["PRECISION"] = np.float16
        elif v in ("SINGLE", "FLOAT32"):
            params["PRECISION"] = np.float32
        elif v in ("DOUBLE", "FLOAT64"):
            params["PRECISION"] = np.float64


def _join(value):
    return value if isinstance(value, str) else "".join(value)


def separated_array_parser(input_array, precision):
    """src/imc_input.jl:97-111: comma-separated numbers, or a tuple literal."""
    joined = _join(input_array)
    if "(" in joined:
        return [ast.literal_eval(joined)]
    return [precision(float(x)) for x in joined.split(",")]


def readInputs(filename):
    """Read an input deck into a dict (src/imc_input.jl:20-95)."""
    params = {}
    current_key = ""
    current_value = []
    in_array = False
    with open(filename, "r") as f:
        for raw in f:
            line = raw.strip()
            if not line or line.startswith("#"):
                continue
            if not in_array and _KEY_RE.match(line):
                parts = line.split("=")
                current_key = parts[0].strip()
                current_value = [parts[1].strip()]
                in_array = False
                if current_key and not current_value[0].startswith("["):
                    params[current_key] = current_value[0]
                elif current_value[0].startswith("["):
                    if not current_value[0].strip().endswith("]"):
                        in_array = True
                    old = current_value[0]
                    current_value = [old.strip("[]")]
                    if not in_array:
                        params[current_key] = current_value
            elif in_array:
                if line.strip().endswith("]"):
                    current_value.append(line.strip("]"))
                    params[current_key] = current_value
                    in_array = False
                else:
                    current_value.append(line.strip())
    precision_set(params)
    prec = params.get("PRECISION", np.float64)
    for key in list(params.keys()):
        if key == "PRECISION":
            continue
        value = params[key]
        if "," in _join(value):
            if key in _NODE_KEYS:
                params[key] = separated_array_parser(value, np.float64)
            else:
                params[key] = separated_array_parser(value, prec)
    return params
