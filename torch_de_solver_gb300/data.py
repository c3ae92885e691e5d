"""Problem definition API: Domain, Conditions, Equation.

Signatures and semantics follow the reference's user API (tedeous/data.py:33-339) so that
problem scripts written for TEDEouS run unchanged:
  * Domain.variable(name, [start, end], n_points) adds n_points + 1 uniform nodes
    (tedeous/data.py:63-67); Domain.build() returns their cartesian product (data.py:83-87).
  * Conditions.* record boundary conditions; build() evaluates every subgrid and every callable
    or scalar boundary value exactly once (tedeous/data.py:241-323).
  * Equation.add appends one equation in operator-dict form (tedeous/data.py:326-339).
Everything here runs on the host at compile time; nothing is on the per-step path.
"""

from copy import deepcopy
from typing import Dict, List, Union

import torch

_DTYPES = {'float32': torch.float32, 'float64': torch.float64, 'float16': torch.float16}


def tensor_dtype(dtype):
    return _DTYPES.get(dtype, dtype)


def unify_operator(equation: dict) -> dict:
    """Per-factor lists for a term's derivative/pow/var; 'var' defaults to 0
    (tedeous/input_preprocessing.py:52-81). The derivative entry is the term's second key."""
    for label in equation:
        term = equation[label]
        key = list(term.keys())[1]
        if 'var' not in term:
            if isinstance(term['pow'], list):
                term['var'] = [0 for _ in term['pow']]
            else:
                term[key] = [term[key]]
                term['pow'] = [term['pow']]
                term['var'] = [0]
            continue
        if not isinstance(term['pow'], list):
            term[key] = [term[key]]
            term['pow'] = [term['pow']]
            term['var'] = [term['var']]
    return equation


class Domain:
    """Uniform grid over named variables."""

    def __init__(self, type: str = 'uniform'):
        self.type = type
        self.variable_dict: Dict[str, torch.Tensor] = {}

    def variable(self, variable_name: str, variable_set: Union[List, torch.Tensor],
                 n_points: Union[None, int], dtype: str = 'float32') -> None:
        dt = tensor_dtype(dtype)
        if isinstance(variable_set, torch.Tensor):
            self.variable_dict[variable_name] = variable_set.detach().cpu().to(dt)
        elif self.type == 'uniform':
            start, end = variable_set
            self.variable_dict[variable_name] = torch.linspace(start, end, n_points + 1, dtype=dt)
        else:
            raise NotImplementedError(f'domain type {self.type!r}')

    def build(self, mode: str, removed_domains: list = None) -> torch.Tensor:
        if mode not in ('NN', 'autograd'):
            raise NotImplementedError(f"mode {mode!r}: only 'NN' and 'autograd' are implemented")
        if removed_domains is not None:
            raise NotImplementedError('removed_domains (CSG grids) are not implemented')
        axes = [v.cpu() for v in self.variable_dict.values()]
        if len(axes) == 1:
            return axes[0].reshape(-1, 1)
        return torch.cartesian_prod(*axes)


class Conditions:
    """Boundary, initial and data conditions."""

    def __init__(self):
        self.conditions_lst: List[dict] = []

    def dirichlet(self, bnd, value, var: int = 0):
        self.conditions_lst.append({'bnd': bnd, 'bop': None, 'bval': value, 'var': var,
                                    'type': 'dirichlet'})

    def operator(self, bnd, operator: dict, value):
        self.conditions_lst.append({'bnd': bnd, 'bop': unify_operator(operator), 'bval': value,
                                    'var': 0, 'type': 'operator'})

    def periodic(self, bnd, operator: dict = None, var: int = 0):
        value = torch.tensor([0.])
        if operator is None:
            self.conditions_lst.append({'bnd': bnd, 'bop': None, 'bval': value, 'var': var,
                                        'type': 'periodic'})
        else:
            self.conditions_lst.append({'bnd': bnd, 'bop': unify_operator(operator),
                                        'bval': value, 'var': 0, 'type': 'periodic'})

    def robin(self, bnd, value, operator: dict = None, var: int = 0):
        self.conditions_lst.append({'bnd': bnd, 'bop': unify_operator(operator), 'bval': value,
                                    'var': var, 'type': 'robin'})

    def data(self, bnd, operator: Union[dict, None], value, var: int = 0):
        if operator is not None:
            operator = unify_operator(operator)
        self.conditions_lst.append({'bnd': bnd, 'bop': operator, 'bval': value, 'var': var,
                                    'type': 'data'})

    @staticmethod
    def _bnd_grid(bnd, variable_dict: dict, dtype) -> torch.Tensor:
        if isinstance(bnd, torch.Tensor):
            g = bnd.detach().cpu().to(dtype)
        else:
            if isinstance(bnd, dict) and list(bnd.keys())[0] == 'circle':
                raise NotImplementedError('CSG circle boundaries are not implemented')
            parts = []
            for name, axis in variable_dict.items():
                spec = bnd[name]
                if isinstance(spec, torch.Tensor):
                    parts.append(spec.detach().cpu().to(dtype).reshape(-1))
                elif isinstance(spec, (float, int)):
                    parts.append(torch.tensor([spec]).to(dtype))
                elif isinstance(spec, list):
                    lo, hi = spec
                    parts.append(axis[(axis >= lo) & (axis <= hi)].to(dtype))
                else:
                    raise TypeError(f'boundary spec for {name!r}: {type(spec)}')
            g = torch.cartesian_prod(*parts).to(dtype)
        if g.dim() == 1:
            g = g.reshape(-1, 1)
        return g

    def build(self, variable_dict: dict) -> Union[None, List[dict]]:
        """Subgrids and boundary values of every condition, evaluated once on the host."""
        if not self.conditions_lst:
            return None
        dtype = next(iter(variable_dict.values())).dtype
        out = []
        for cond in deepcopy(self.conditions_lst):
            if cond['type'] == 'periodic':
                cond['bnd'] = [self._bnd_grid(b, variable_dict, dtype) for b in cond['bnd']]
            else:
                cond['bnd'] = self._bnd_grid(cond['bnd'], variable_dict, dtype)
            v = cond['bval']
            if isinstance(v, torch.Tensor):
                cond['bval'] = v.detach().cpu().to(dtype)
            elif isinstance(v, (float, int)):
                cond['bval'] = (torch.ones_like(cond['bnd'][:, 0]) * v).to(dtype)
            elif callable(v):
                cond['bval'] = torch.as_tensor(v(cond['bnd'])).detach().cpu().to(dtype)
            out.append(cond)
        return out


class Equation:
    """List of equations in operator-dict form."""

    def __init__(self):
        self.equation_lst: List[dict] = []

    def add(self, eq: dict):
        self.equation_lst.append(eq)
