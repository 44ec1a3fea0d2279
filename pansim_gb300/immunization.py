"""Immunization options on the host side of the C ABI.

`options(...)` takes the reference's command-line options
(include/immunization.h:96-133, same names and defaults) and packs them into
the psim_immunization struct for psim_immunization_init.  Weekly schedules
(the file forms of --immunizationsPerWeek / --boostersPerWeek) are given as
lists: one list of weekly doses, and per booster round a list of weekly
doses plus its ten age-group percentages.
"""
from . import cabi

DEFAULTS = dict(
    immunizationStart=96,
    boosterStart="315",
    immunizationOrder="1,2,3,4,5,6,0,0,7,8",
    vaccinationGroupLevel="0.9,0.85,0.9,0.82,0.8,0.75,0.8,0.67,0.4,0.2",
    protectionInfection="0.85,0.5,0.77,0.4,0.85,0.63,0.9,0.65,0.92,0.7",
    protectionInfectionWaning="0.003,0.006,0.01,0.02,0.005,0.02,0.002,0.004,0.002,0.004",
    protectionSymptomatic="0.9,0.55,0.8,0.6,0.95,0.69,0.92,0.7,0.94,0.77",
    protectionSymptomaticWaning="0.003,0.006,0.01,0.02,0.005,0.02,0.002,0.004,0.002,0.004",
    protectionHospitalization="0.92,0.85,0.95,0.9,0.97,0.92,0.974,0.93,0.98,0.97",
    protectionHospitalizationWaning="0.0021,0.006,0.006,0.006,0.003,0.003,0.0014,0.003,0.0014,0.003",
    variantSimilarity="0,0,0,1,1,1,1",
    variantSimilarMultiplier="0.0,0.0,0.0,0.0,0.0,0.0,0.0",
)


def _split(v, conv):
    if isinstance(v, str):
        return [conv(x) for x in v.split(",") if x.strip()]
    return [conv(x) for x in v]


def options(immunizations_per_week=0, boosters_per_week=None, **kw):
    """psim_immunization from the reference's options.

    immunizations_per_week: a number (doses per week, --immunizationsPerWeek N)
        or a list of weekly doses (the file form).
    boosters_per_week: None, a number (--boostersPerWeek N; the reference then
        reads no age-group percentages, so give them with booster_age_percent)
        or a list with one (weekly doses, ten age-group percentages) pair per
        booster round.
    Other keyword arguments use the reference's option names (DEFAULTS).
    """
    o = dict(DEFAULTS)
    o.update(kw)
    p = cabi.PsimImmunization()
    p.start_after_day = int(o["immunizationStart"])
    if isinstance(immunizations_per_week, (list, tuple)):
        if len(immunizations_per_week) > cabi.PSIM_IMM_MAX_WEEKS:
            raise ValueError("more weeks than PSIM_IMM_MAX_WEEKS")
        p.n_vacc_weeks = len(immunizations_per_week)
        for w, x in enumerate(immunizations_per_week):
            p.vacc_per_week[w] = float(x)
    else:
        p.daily_doses = int(immunizations_per_week) // 7
    starts = _split(str(o["boosterStart"]), int)
    if len(starts) > cabi.PSIM_IMM_MAX_ROUNDS:
        raise ValueError("more booster rounds than PSIM_IMM_MAX_ROUNDS")
    p.n_booster_rounds = len(starts)
    for r, s in enumerate(starts):
        p.booster_start_after_day[r] = s
    if isinstance(boosters_per_week, (list, tuple)):
        if len(boosters_per_week) != len(starts):
            raise ValueError("booster rounds size mismatch")
        for r, (weeks, pct) in enumerate(boosters_per_week):
            p.n_booster_weeks[r] = len(weeks)
            for w, x in enumerate(weeks):
                p.booster_per_week[r][w] = float(x)
            for g, x in enumerate(pct):
                p.booster_age_percent[r][g] = float(x)
    elif boosters_per_week is not None:
        p.daily_boosters = int(boosters_per_week) // 7
        pct = o.get("booster_age_percent", [1.0] * 10)
        for r in range(len(starts)):
            for g in range(10):
                p.booster_age_percent[r][g] = float(pct[g])
    order = _split(o["immunizationOrder"], int)
    level = _split(o["vaccinationGroupLevel"], float)
    if len(order) != cabi.PSIM_IMM_CATEGORIES:
        raise ValueError("immunizationOrder must have exactly 10 values")
    for g in range(10):
        p.order[g] = order[g]
        p.group_level[g] = level[g]
    for name, field in [("protectionInfection", "protection_infection"),
                        ("protectionInfectionWaning", "protection_infection_waning"),
                        ("protectionSymptomatic", "protection_symptomatic"),
                        ("protectionSymptomaticWaning", "protection_symptomatic_waning"),
                        ("protectionHospitalization", "protection_hospitalization"),
                        ("protectionHospitalizationWaning", "protection_hospitalization_waning")]:
        vals = _split(o[name], float)
        arr = getattr(p, field)
        for j in range(10):
            arr[j] = vals[j]
    sim = _split(o["variantSimilarity"], int)
    vsm = _split(o["variantSimilarMultiplier"], float)
    for v in range(cabi.PSIM_MAX_STRAINS):
        p.variant_similarity[v] = sim[v] if v < len(sim) else 0
        p.variant_similar_multiplier[v] = vsm[v] if v < len(vsm) else 0.0
    return p
