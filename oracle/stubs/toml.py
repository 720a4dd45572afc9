"""``toml`` stand-in on top of ``tomllib`` (test infrastructure only): ``load``
reads a file, ``dumps`` writes the flat key = value form the reference's
metadata files use."""
import tomllib


def load(path):
    with open(path, "rb") as fh:
        return tomllib.load(fh)


def _fmt(value):
    if isinstance(value, bool):
        return "true" if value else "false"
    if isinstance(value, str):
        return '"' + value.replace('"', '\\"') + '"'
    if isinstance(value, (list, tuple)):
        return "[ " + ", ".join(_fmt(v) for v in value) + ",]"
    if isinstance(value, float):
        # toml prints floats with one exponent digit where it can (1e-5)
        return repr(value).replace("e+0", "e+").replace("e-0", "e-")
    return repr(value)


def dumps(data):
    return "".join(f"{k} = {_fmt(v)}\n" for k, v in data.items())
