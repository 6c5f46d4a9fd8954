"""The time loop of the reference's model program around the GPU step.

`run` is `ccsm.F90:40-63` with the step replaced by the library: initial mass and
energy, `nsteps` steps of RK4 / RK3_TVD, and at every history time the state handed
to an output callback (the place of `history_write_stat`) and the mass and energy
change ratios (MCR, ECR) printed in the reference's format.  The device keeps the
state between outputs, so the steps between two outputs are one `ccs_step(h, k)`
call (graph replays, no host round trip) instead of the reference's per-step copy.

Time settings follow `parameters_mod.F90`: the namelist group `time_settings`
(:87-92) and its defaults (:118-128), `total_run_time` (:135) and
`nsteps = total_run_time / dt` truncated to an integer (:149).  An output happens
after step `it` when `mod(it*dt, history_interval) == 0` and
`it*dt >= history_interval` (`ccsm.F90:55`), both in double precision as the
reference evaluates them.

The reference computes the energy at an output time from `stat(old)`, the state
before the last step (`ccsm.F90:60`; the mass uses `stat(new)`).  `run` reproduces
that by default; `energy_of_new_state=True` takes the energy of the output state
instead.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Callable


@dataclass
class TimeSettings:
    """parameters_mod.F90:9-14 with the defaults of :118-128."""
    dt: float = 300.0
    run_days: int = 1
    run_hours: int = 0
    run_minutes: int = 0
    run_seconds: int = 0
    history_interval: int = 360
    integral_scheme: str = "RK4"

    @property
    def total_run_time(self) -> int:
        return self.run_days * 86400 + self.run_hours * 3600 + self.run_minutes * 60 + self.run_seconds

    @property
    def nsteps(self) -> int:
        return int(self.total_run_time / self.dt)

    @property
    def total_output_num(self) -> int:
        return int(self.nsteps * self.dt / self.history_interval)


def output_steps(ts: TimeSettings) -> list[int]:
    """The steps after which ccsm.F90:55 writes output."""
    hi = float(ts.history_interval)
    out = []
    for it in range(1, ts.nsteps + 1):
        t = it * ts.dt
        if math.fmod(t, hi) == 0.0 and t >= hi:
            out.append(it)
    return out


@dataclass
class OutputRecord:
    output_idx: int
    step: int
    mcr: float  # (mass - mass0) / mass0
    ecr: float  # (energy - energy0) / energy0
    courant: float | None = None  # Courant number of the output state (with max_courant)


def run(stepper, ts: TimeSettings, on_output: Callable | None = None, energy_of_new_state: bool = False,
        log: Callable[[str], None] | None = print, check: bool = True,
        max_courant: float | None = None) -> list[OutputRecord]:
    """Advances `stepper` (a model.Stepper whose state is set) through the run of
    `ts`; calls on_output(output_idx, state) at every history time with the state
    as ccs_get_state returns it (sphere winds included); returns the MCR/ECR records.
    With `check`, every output time also runs the health check (ccs_check_state) and
    a state with non-positive depth or non-finite wind stops the run with
    FloatingPointError (the reference has no such check and carries on with NaNs).
    With `max_courant`, every output time also takes the state's Courant number
    (ccs_courant) into its record and stops the run with FloatingPointError above
    that bound (the reference's dt is a namelist constant that nothing checks)."""
    if ts.integral_scheme not in ("RK4", "RK3_TVD"):
        raise ValueError(f"integral_scheme {ts.integral_scheme!r}")
    mass0, energy0 = stepper.diag()
    if on_output is not None:
        on_output(1, stepper.get_state())
    if log:
        log(f" output index/total, MCR, ECR : {0} / {ts.total_output_num}   0.0 0.0")
    records = []
    done = 0
    for k, it in enumerate(output_steps(ts)):
        ahead = it - done
        if energy_of_new_state:
            stepper.step(ahead)
            mass, energy = stepper.diag()
        else:
            if ahead > 1:
                stepper.step(ahead - 1)
            energy = stepper.diag()[1]  # stat(old): the state before step `it`
            stepper.step(1)
            mass = stepper.diag()[0]
        done = it
        idx = k + 2
        if check:
            nbad = stepper.check_state()
            if nbad:
                raise FloatingPointError(f"step {it}: {nbad} cells with non-positive depth or non-finite wind")
        courant = None
        if max_courant is not None:
            courant = stepper.courant()
            if not courant <= max_courant:
                raise FloatingPointError(f"step {it}: Courant number {courant:.4g} above {max_courant}")
        if on_output is not None:
            on_output(idx, stepper.get_state())
        rec = OutputRecord(idx, it, (mass - mass0) / mass0, (energy - energy0) / energy0, courant)
        records.append(rec)
        if log:
            log(f" output index/total, MCR, ECR : {idx - 1} / {ts.total_output_num}   {rec.mcr!r} {rec.ecr!r}")
    if ts.nsteps > done:
        stepper.step(ts.nsteps - done)
    return records
