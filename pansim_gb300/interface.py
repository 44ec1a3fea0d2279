"""The reference's day-at-a-time binding, pyPanSim.SimulatorInterface
(matlab/mexPanSim.cpp:57-127, pybind11 module :210-219), over the library.

initSimulation takes a population snapshot (pansim_gb300.snapshot.Snapshot,
for instance from pansim_gb300.reference_inputs.load of the reference's
input files) and the optional closure rules, immunization and otherDisease
settings, where the reference parses its command-line options.  runForDay
follows Simulation::runForDay (simulation.h:928-956):

1. the day's flags (Simulation::processFlags, :779-897);
2. the statistics of the midnight before, the closure rules on them, and
   planLocations;
3. the day's timesteps (one day graph);
4. at the midnight after: testing, progression, immunization, otherDisease,
   and that midnight's statistics row, which it returns.

A context holding several replicas (pansim_gb300.snapshot.concat) runs them
all with the same flags; runForDayBatch returns every replica's row.
Unknown flags are ignored, as processFlags ignores them.
"""
from pansim_gb300.native import GpuSim

# processFlags' testing probabilities (random, home, work, school, hospital,
# nursery home: TestingPolicy::updateTestingProbs, testingPolicies.h:328-338)
TESTING_FLAGS = {
    "TPdef": "0.00005,0.01,0.0005,0.0005,0.005,0.05",
    "TP015": "0.00005,0.2,0.04,0.04,0.005,0.05",
    "TP035": "0.00005,1.0,0.2,0.2,0.005,0.05",
}
TESTING_KEYS = ["t_random", "t_home", "t_work", "t_school", "t_hospital", "t_nursery"]
# the location types that "PLNONE" / "PL0" open / close (simulation.h:796, :813)
FLAG_CLOSE_TYPES = (5, 6, 22, 44)
SCHOOL_AGE_FLAGS = {"SONONE": 99, "SO12": 12, "SO3": 3}
QUARANTINE_FLAGS = {"QU0": 0, "QU1": 1, "QU2": 2, "QU3": 3}


def testing_probs(text):
    """updateTestingProbs: the leading comma-separated values, in order."""
    vals = [float(x) for x in text.split(",") if x.strip() != ""]
    return dict(zip(TESTING_KEYS, vals))


def parse_flags(flags, time_step, mask):
    """The actions of processFlags for `flags`, in order, given the model's
    timestep (minutes) and the current mask value.  Returns (actions, mask):
    each action is ("params", {name: value}), ("types_open", types, open) or
    ("weights", coef, divide)."""
    actions = []
    for flag in flags:
        prefix = flag[:2]
        if prefix == "TP":
            if flag in TESTING_FLAGS:
                actions.append(("params", testing_probs(TESTING_FLAGS[flag])))
        elif prefix == "PL":
            if flag == "PLNONE":
                actions.append(("types_open", FLAG_CLOSE_TYPES, True))
            elif flag == "PL0":
                actions.append(("types_open", FLAG_CLOSE_TYPES, False))
        elif prefix == "CF":
            # toggleCurfew (simulation.h:958-963): minutes, converted to
            # timesteps by the movement policy
            if flag == "CFNONE":
                actions.append(("params", dict(enable_curfew=0, curfew_begin=0, curfew_end=0)))
            elif flag == "CF2000-0500":
                actions.append(("params", dict(enable_curfew=1, curfew_begin=(20 * 60) // time_step,
                                               curfew_end=(5 * 60) // time_step)))
        elif prefix == "SO":
            if flag in SCHOOL_AGE_FLAGS:
                actions.append(("params", dict(school_age_restriction=SCHOOL_AGE_FLAGS[flag])))
        elif prefix == "QU":
            if flag in QUARANTINE_FLAGS:
                actions.append(("params", dict(quarantine_policy=QUARANTINE_FLAGS[flag])))
        elif prefix == "MA":
            if flag == "MA1.0" and mask != 1.0:
                actions.append(("weights", mask, True))
                mask = 1.0
            elif flag == "MA0.8" and mask != 0.8:
                mask = 0.8
                actions.append(("weights", 0.8, False))
    return actions, mask


class SimulatorInterface:
    """pyPanSim.SimulatorInterface: initSimulation, then runForDay once per
    simulated day."""

    def __init__(self):
        self.sim = None
        self.day = 0
        self.mask = 1.0
        self._closures = self._imm = self._od = False

    def initSimulation(self, snapshot, closure_rules=None, closure_header=None, enable_closures=True,
                       immunization=None, other_disease=None, device=0):
        self.sim = GpuSim(snapshot, device=device)
        self._closures = closure_rules is not None
        if self._closures:
            self.sim.closures_init(closure_rules, closure_header, enable_closures)
        self._imm = immunization is not None
        if self._imm:
            self.sim.immunization_init(immunization)
        self._od = other_disease is not None
        if self._od:
            self.sim.other_disease_init(other_disease)
        self.day = 0
        self.mask = 1.0

    def apply_flags(self, flags):
        snap = self.sim.snap
        actions, self.mask = parse_flags(flags, int(snap.params["time_step"]), self.mask)
        params_changed = False
        for act in actions:
            if act[0] == "params":
                snap.params.update(act[1])
                params_changed = True
            elif act[0] == "types_open":
                self.sim.set_types_open(act[1], act[2])
            else:
                self.sim.scale_location_weights(act[1], act[2])
        if params_changed:
            self.sim.set_params()

    def runForDayBatch(self, flags):
        """One day for every replica; returns each replica's statistics row
        of the midnight after the day (an empty list before initSimulation,
        as the reference returns an empty vector)."""
        if self.sim is None:
            return []
        self.apply_flags(flags)
        sim, spd = self.sim, self.sim.snap.steps_per_day
        t = self.day * spd
        rows = sim.stats(t)
        if self._closures:
            sim.closures_midnight(t, rows[0])
        sim.plan(t)
        sim.run_steps(self.day)
        t_end = t + spd
        if int(sim.snap.params.get("testing_enabled", 0)):
            sim.test(t_end)
        sim.progress(t_end)
        if self._imm:
            sim.immunize(t_end)
        if self._od:
            sim.other_disease(t_end)
        rows = sim.stats(t_end)
        self.day += 1
        return [[int(x) for x in r.v[: r.n]] for r in rows]

    def runForDay(self, flags):
        """One day; replica 0's statistics row."""
        rows = self.runForDayBatch(flags)
        return rows[0] if rows else []
