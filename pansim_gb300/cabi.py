"""ctypes mirrors of the structs in include/pansim_gb300.h.

Field order and types must match the header exactly; tests compare the sizes
with the ones the compiled library reports (psim_abi_sizes).
"""
import ctypes as C

P = C.c_void_p
PSIM_MAX_STRAINS = 7
PSIM_MAX_BANDS = 16
PSIM_STATS_MAX = 64


class PsimModel(C.Structure):
    _fields_ = [
        ("n_states", C.c_uint32), ("n_variants", C.c_uint32), ("n_prog", C.c_uint32),
        ("n_agent_types", C.c_uint32), ("n_trans", C.c_uint32), ("n_events", C.c_uint32),
        ("first_infected_state", C.c_uint32), ("noncovid_dead_state", C.c_uint32),
        ("dead_state", C.c_uint32), ("pad0", C.c_uint32),
        ("state_wb", P), ("state_infectious", P), ("state_susceptible", P), ("state_infected", P),
        ("state_acc_pcr", P), ("state_acc_antigen", P),
        ("variant_multiplier", P), ("prog_scaling", P), ("death_scaling", P),
        ("tr_bad_begin", P), ("tr_bad_count", P), ("tr_neu_begin", P), ("tr_neu_count", P),
        ("tr_next", P), ("tr_chance", P),
        ("len_avg", P), ("len_max", P), ("len_p", P),
        ("event_offset", P), ("ev_loc_type", P), ("ev_chance", P), ("ev_start", P), ("ev_end", P),
        ("ev_duration", P),
    ]


AGENT_PTR_FIELDS = [
    "type", "age", "band", "prog_id", "symptom_scaling", "loc_offset", "poss_loc", "poss_type",
    "location", "steps_until_move", "state", "days", "variant", "infectious", "susceptible",
    "diagnosed", "quarantined", "stayed_home", "no_work", "last_test",
    "st_infected_ts", "st_infected_loc", "st_worst_ts", "st_worst_end_ts", "st_diagnosed_ts",
    "st_quarantined_ts", "st_quarantined_until", "st_days_in_quarantine", "st_hospitalized_ts",
    "st_hospitalized_until", "st_immunization_ts", "st_recovered_ts", "st_variant_mask",
    "st_immunization_count", "st_infected_count", "st_worst_state", "precond", "imm_round", "symptom_scaling_v",
    "sex",
]


class PsimAgents(C.Structure):
    _fields_ = [("n", C.c_uint32), ("n_poss", C.c_uint32)] + [(f, P) for f in AGENT_PTR_FIELDS]


LOC_PTR_FIELDS = ["type", "infectiousness", "open", "essential", "closed_until", "quarantine_until",
                  "schools", "classrooms", "classroom_offsets"]


class PsimLocations(C.Structure):
    _fields_ = [("n", C.c_uint32), ("n_schools", C.c_uint32), ("n_classrooms", C.c_uint32),
                ("pad0", C.c_uint32)] + [(f, P) for f in LOC_PTR_FIELDS]


PARAM_U32 = ["time_step", "start_day", "start_date", "home_type", "work_type", "school_type",
             "classroom_type", "hospital_type", "doctor_type", "public_type", "nursery_type",
             "cemetery_loc", "quarantine_policy", "quarantine_length", "enable_curfew", "curfew_begin",
             "curfew_end", "school_age_restriction", "holiday_mode", "quarantine_immune",
             "lockdown_nonvacc", "testing_enabled", "testing_delay", "use_pcr", "n_bands", "tracked",
             "pad0"]


class PsimParams(C.Structure):
    _fields_ = ([(f, C.c_uint32) for f in PARAM_U32] +
                [("k", C.c_double), ("c0", C.c_double), ("trunc", C.c_double),
                 ("d_offset0", C.c_int32), ("d_offset1", C.c_int32), ("d_peak_offset", C.c_int32),
                 ("n_d_offset", C.c_int32),
                 ("t_random", C.c_double), ("t_home", C.c_double), ("t_work", C.c_double),
                 ("t_school", C.c_double), ("t_hospital", C.c_double), ("t_nursery", C.c_double),
                 ("seed", C.c_uint64), ("sigma_band", C.c_float * PSIM_MAX_BANDS)])


class PsimReplicas(C.Structure):
    _fields_ = [("n", C.c_uint32), ("pad0", C.c_uint32), ("agent_offset", P), ("loc_offset", P),
                ("seed", P), ("k", P), ("cemetery", P)]


class PsimDayStats(C.Structure):
    _fields_ = [("n", C.c_uint32), ("new_infections", C.c_uint32), ("v", C.c_uint32 * PSIM_STATS_MAX),
                ("variant_counts", C.c_uint32 * PSIM_MAX_STRAINS), ("expected_new_infections", C.c_double)]


class PsimTuning(C.Structure):
    _fields_ = [("agg_count", C.c_uint32), ("agg_slot", C.c_uint32), ("blocks_per_sm", C.c_uint32),
                ("variant", C.c_uint32), ("scan_items", C.c_uint32), ("scan_mode", C.c_uint32)]


PSIM_IMM_CATEGORIES = 10
PSIM_IMM_MAX_ROUNDS = 8
PSIM_IMM_MAX_WEEKS = 160


class PsimImmunization(C.Structure):
    _fields_ = [("start_after_day", C.c_uint32), ("daily_doses", C.c_uint32), ("n_vacc_weeks", C.c_uint32),
                ("n_booster_rounds", C.c_uint32), ("daily_boosters", C.c_uint32), ("pad0", C.c_uint32),
                ("vacc_per_week", C.c_float * PSIM_IMM_MAX_WEEKS),
                ("booster_start_after_day", C.c_int32 * PSIM_IMM_MAX_ROUNDS),
                ("n_booster_weeks", C.c_uint32 * PSIM_IMM_MAX_ROUNDS),
                ("booster_per_week", (C.c_float * PSIM_IMM_MAX_WEEKS) * PSIM_IMM_MAX_ROUNDS),
                ("booster_age_percent", (C.c_float * 10) * PSIM_IMM_MAX_ROUNDS),
                ("order", C.c_int32 * PSIM_IMM_CATEGORIES), ("group_level", C.c_float * PSIM_IMM_CATEGORIES),
                ("protection_infection", C.c_float * 10), ("protection_infection_waning", C.c_float * 10),
                ("protection_symptomatic", C.c_float * 10), ("protection_symptomatic_waning", C.c_float * 10),
                ("protection_hospitalization", C.c_float * 10),
                ("protection_hospitalization_waning", C.c_float * 10),
                ("variant_similarity", C.c_int32 * PSIM_MAX_STRAINS),
                ("variant_similar_multiplier", C.c_float * PSIM_MAX_STRAINS)]


class PsimOtherDisease(C.Structure):
    _fields_ = [("enabled", C.c_uint32), ("due_with_covid", C.c_uint32), ("n_targets", C.c_uint32),
                ("pad0", C.c_uint32), ("total_hospitalizations", P)]


def other_disease_options(enabled=1, due_with_covid=0, total_hospitalizations=None):
    """psim_other_disease for --otherDisease, --dueWithCOVID and the per-day
    --totalHospitalizations targets (None: the yearly multipliers)."""
    import numpy as np
    od = PsimOtherDisease()
    od.enabled = int(enabled)
    od.due_with_covid = int(due_with_covid)
    if total_hospitalizations is not None and len(total_hospitalizations):
        arr = np.ascontiguousarray(total_hospitalizations, dtype=np.int32)
        od._targets = arr  # keeps the buffer alive with the struct
        od.n_targets = len(arr)
        od.total_hospitalizations = arr.ctypes.data
    return od


PSIM_CLOSURE_MAX_TYPES = 10


class PsimClosureRule(C.Structure):
    _fields_ = [("name", C.c_char * 64), ("condition_type", C.c_char * 32), ("threshold", C.c_double),
                ("threshold2", C.c_double), ("parameter", C.c_char * 64), ("close_after", C.c_int32),
                ("open_after", C.c_int32), ("n_types", C.c_uint32), ("types", C.c_int32 * PSIM_CLOSURE_MAX_TYPES)]


ABI_STRUCTS = [PsimModel, PsimAgents, PsimLocations, PsimParams, PsimReplicas, PsimDayStats]
