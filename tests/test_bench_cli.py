"""The bench's command line: every option the bench reads exists with its default, so a
plain `python bench.py` (no options) parses and dispatches (host only, no GPU)."""
import ast
import importlib.util
import os

from _lib import ROOT


def _bench():
    spec = importlib.util.spec_from_file_location("bench_cli", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_every_option_read_has_a_default():
    bench = _bench()
    args = bench.make_parser().parse_args([])
    with open(os.path.join(ROOT, "bench.py")) as fh:
        tree = ast.parse(fh.read())
    read = {n.attr for n in ast.walk(tree)
            if isinstance(n, ast.Attribute) and isinstance(n.value, ast.Name) and n.value.id == "args"}
    missing = sorted(a for a in read if not hasattr(args, a))
    assert not missing, missing
    assert args.gpus == 1 and args.steps >= 1 and args.warmup >= 3
    assert not args.config3 and args.config4 == 0 and args.impl == "gb300"


def test_sweep_and_refined_legs_parse():
    args = _bench().make_parser().parse_args(["--config4", "256", "--config3"])
    assert args.config4 == 256 and args.config3
