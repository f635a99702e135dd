"""Data directories, the counterpart of `rc[:paths]` (src/PorousMaterials.jl:29-36)."""
from __future__ import annotations

from pathlib import Path

rc: dict = {"paths": {}}


def set_paths(root: str | Path) -> None:
    root = Path(root)
    rc["paths"].update({
        "crystals": str(root / "crystals"),
        "forcefields": str(root / "forcefields"),
        "molecules": str(root / "molecules"),
        "grids": str(root / "grids"),
        "simulations": str(root / "simulations"),
    })


set_paths(Path.cwd() / "data")
