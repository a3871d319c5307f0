"""Output / simulation keyword defaults and checks (utils.py:12-146)."""
from __future__ import annotations

from typing import Dict


def default_outputkw() -> Dict:
    return {"file": "topopt", "display": True, "export": True, "write_log": True,
            "profile": False, "output_movie": False, "verbosity": 20}


def check_output_kw(output_kw: Dict) -> None:
    """Insert missing keys from the defaults (in place)."""
    for key, val in default_outputkw().items():
        output_kw.setdefault(key, val)


def check_simulation_params(simulation_kw: Dict) -> None:
    admissible = {"grid": ["regular"], "element order": [1], "meshfile": [None]}
    for key, allowed in admissible.items():
        if simulation_kw[key] not in allowed:
            raise ValueError(f"{key} must be one of those: {allowed}")
