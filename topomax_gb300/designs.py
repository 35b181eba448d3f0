"""Design description: the JSON format of the reference's ``designs/*.json``.

Same schema and error behaviour as ``designs/definitions.py:22-223`` and
``designs/design_parser.py:12-34`` (one top-level key naming the problem,
``domain_parameters`` and ``problem_parameters``).  Elasticity designs may
carry an extra ``fixed_points`` list of clamped vertices (x, y); it has no
counterpart in the reference, whose clamping is whole sides only.
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field
from enum import Enum, auto


def to_2_tuple(ray):
    if len(ray) != 2:
        raise ValueError("Got array that should have had 2 elements, "
                         f"but had {len(ray)} instead: '{ray}'")
    return (ray[0], ray[1])


class Side(Enum):
    LEFT = auto()
    RIGHT = auto()
    TOP = auto()
    BOTTOM = auto()

    @classmethod
    def get_all(cls):
        return [cls.LEFT, cls.RIGHT, cls.TOP, cls.BOTTOM]

    @classmethod
    def from_string(cls, string: str):
        table = {"Left": cls.LEFT, "Right": cls.RIGHT, "Top": cls.TOP, "Bottom": cls.BOTTOM}
        if string in table:
            return table[string]
        raise ValueError(f"Malformed side: '{string}'\nLegal sides "
                         "are: 'Left', ''Right', 'Top' or 'Bottom'")

    @property
    def mask(self) -> int:
        return {Side.LEFT: 1, Side.RIGHT: 2, Side.TOP: 4, Side.BOTTOM: 8}[self]


class ProblemType(Enum):
    FLUID = auto()
    ELASTICITY = auto()

    @classmethod
    def from_string(cls, problem: str):
        if problem == "Fluid":
            return cls.FLUID
        if problem == "Elasticity":
            return cls.ELASTICITY
        raise ValueError(f"Malformed problem: '{problem}'\nLegal problems "
                         "are: 'Fluid' and 'Elasticity'")


@dataclass
class CircularRegion:
    center: tuple
    radius: float

    @classmethod
    def from_dict(cls, d: dict):
        return cls(to_2_tuple(d["center"]), d["radius"])


@dataclass
class Force:
    region: CircularRegion
    value: tuple

    @classmethod
    def from_dict(cls, d: dict):
        return cls(CircularRegion.from_dict(d["region"]), to_2_tuple(d["value"]))


@dataclass
class Traction:
    side: Side
    center: float
    length: float
    value: tuple

    @classmethod
    def from_dict(cls, d: dict):
        return cls(Side.from_string(d["side"]), d["center"], d["length"], to_2_tuple(d["value"]))

    def to_tuple(self):
        return (self.side, self.center, self.length, self.value)


@dataclass
class ElasticityParameters:
    fixed_sides: list
    body_force: Force | None
    tractions: list | None
    filter_radius: float
    young_modulus: float
    poisson_ratio: float
    fixed_points: list = field(default_factory=list)

    @classmethod
    def from_dict(cls, d: dict):
        fixed_sides = [Side.from_string(s) for s in d["fixed_sides"]]
        body_force = Force.from_dict(d["body_force"]) if d.get("body_force") is not None else None
        tractions = None
        if d.get("tractions") is not None:
            tractions = [Traction.from_dict(t) for t in d["tractions"]]
        points = [to_2_tuple(p) for p in d.get("fixed_points") or []]
        return cls(fixed_sides, body_force, tractions, d["filter_radius"], d["young_modulus"],
                   d["poisson_ratio"], points)


@dataclass
class Flow:
    """A parabolic in- or outflow on one side (designs/definitions.py:105-121)."""
    side: Side
    center: float
    length: float
    rate: float

    @classmethod
    def from_dict(cls, d: dict):
        return cls(Side.from_string(d["side"]), d["center"], d["length"], d["rate"])

    def to_tuple(self):
        return (self.side, self.center, self.length, self.rate)


@dataclass
class FluidParameters:
    flows: list
    viscosity: float

    @classmethod
    def from_dict(cls, d: dict):
        return cls([Flow.from_dict(f) for f in d["flows"]], d["viscosity"])


@dataclass
class DomainParameters:
    width: float
    height: float
    problem: ProblemType
    fem_step_size: float
    dem_step_size: float
    penalties: list
    volume_fraction: float

    @classmethod
    def from_dict(cls, problem: str, d: dict):
        return cls(d["width"], d["height"], ProblemType.from_string(problem), d["fem_step_size"],
                   d["dem_step_size"], d["penalties"], d["volume_fraction"])


def parse_design_dict(design_dict: dict):
    keys = list(design_dict.keys())
    if len(keys) > 1:
        raise ValueError(f"Malformed design: got more than one key: {keys}")
    key = keys[0]
    domain = DomainParameters.from_dict(key, design_dict[key]["domain_parameters"])
    params = design_dict[key]["problem_parameters"]
    if domain.problem == ProblemType.FLUID:
        return domain, FluidParameters.from_dict(params)
    if domain.problem == ProblemType.ELASTICITY:
        return domain, ElasticityParameters.from_dict(params)
    raise ValueError(f"Unknown problem: {domain.problem}")


def parse_design(filename: str):
    with open(filename, "rb") as f:
        return parse_design_dict(json.load(f))
