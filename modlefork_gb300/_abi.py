"""ctypes mirror of include/mgpu_modle.h (the C ABI of the GB300 epoch engine).

The structs below follow the header field by field; ``check_layout`` compares their sizes
with the values the compiled library reports, so a drift between the two fails loudly.
"""

import ctypes as C

MGPU_OK = 0
MGPU_ERR_INVALID_ARG = -1
MGPU_ERR_CUDA = -2
MGPU_ERR_TIMEOUT = -3
MGPU_ERR_OVERFLOW = -4
MGPU_ERR_UNSUPPORTED = -5
MGPU_ERR_NO_DEVICE = -6
MGPU_ERR_OUT_OF_MEMORY = -7
MGPU_ERR_INTERNAL = -8
MGPU_NOALLOC_SCRATCH_BYTES = 8 << 20
MGPU_NOALLOC_MAX_CELLS = 16384

STATUS_NAMES = {
    0: "MGPU_OK", -1: "MGPU_ERR_INVALID_ARG", -2: "MGPU_ERR_CUDA", -3: "MGPU_ERR_TIMEOUT",
    -4: "MGPU_ERR_OVERFLOW", -5: "MGPU_ERR_UNSUPPORTED", -6: "MGPU_ERR_NO_DEVICE",
    -7: "MGPU_ERR_OUT_OF_MEMORY", -8: "MGPU_ERR_INTERNAL",
}

CS_NOISIFY, CS_TAD, CS_LOOP = 1, 2, 4
DIR_REV, DIR_FWD = 1, 2
COLL_COLLISION, COLL_CHROM_BOUNDARY, COLL_LEF_BAR = 0x10, 0x08, 0x04
COLL_LEF_LEF_PRIMARY, COLL_LEF_LEF_SECONDARY = 0x02, 0x01

PHASES = {
    "BIND": 1, "RANK": 2, "ADJUST_AND_CLAMP": 3, "GENERATE_MOVES": 4,
    "PROCESS_COLLISIONS": 5, "FIX_SECONDARY": 6, "DETECT_LEF_BAR": 7, "LEF_LEF": 8,
    "DETECT_PRIMARY": 9, "EXTRUDE": 10, "RELEASE": 11, "BARRIER_NEXT": 12,
    "BARRIER_INIT": 13, "DETECT_BOUNDARIES": 14, "CORRECT_LEF_BAR": 15, "CORRECT_PRIMARY": 16,
}

u32, u64, f64 = C.c_uint32, C.c_uint64, C.c_double


class Config(C.Structure):
    _fields_ = [
        ("target_simulation_epochs", u64), ("target_contact_density", f64),
        ("stop_on_epochs", u32),
        ("bin_size", u64), ("diagonal_width", u64), ("contact_sampling_strategy", u32),
        ("tad_to_loop_contact_ratio", f64), ("genextreme_mu", f64), ("genextreme_sigma", f64),
        ("genextreme_xi", f64),
        ("fwd_extrusion_speed", u64), ("rev_extrusion_speed", u64),
        ("fwd_extrusion_speed_std", f64), ("rev_extrusion_speed_std", f64),
        ("number_of_lefs_per_mbp", f64), ("prob_of_lef_release", f64),
        ("prob_of_lef_release_burnin", f64), ("avg_lef_processivity", u64),
        ("contact_sampling_interval", u64),
        ("extrusion_barrier_occupancy", f64), ("barrier_occupied_stp", f64),
        ("barrier_not_occupied_stp", f64),
        ("hard_stall_lef_stability_multiplier", f64), ("soft_stall_lef_stability_multiplier", f64),
        ("probability_of_extrusion_unit_bypass", f64), ("lef_bar_major_collision_pblock", f64),
        ("lef_bar_minor_collision_pblock", f64),
        ("num_cells", u64), ("seed", u64), ("probability_normalization_factor", u64),
        ("normalize_probabilities", u32),
        ("skip_burnin", u32), ("burnin_history_length", u64),
        ("burnin_smoothing_window_size", u64), ("min_burnin_epochs", u64),
        ("max_burnin_epochs", u64), ("burnin_target_epochs_for_lef_activation", u64),
        ("burnin_speed_coefficient", f64), ("fwd_extrusion_speed_burnin", u64),
        ("rev_extrusion_speed_burnin", u64),
        ("rev_speed_set", u32), ("fwd_speed_set", u32), ("occupancy_set", u32),
        ("track_1d_lef_position", u32), ("log_model_internal_state", u32),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class Chrom(C.Structure):
    _fields_ = [("name", C.c_char_p), ("name_len", u64), ("size", u64), ("start", u64),
                ("end", u64)]


class Barrier(C.Structure):
    _fields_ = [("pos", u64), ("stp_active", f64), ("stp_inactive", f64),
                ("blocking_dir", u32), ("reserved", u32)]


class CellStats(C.Structure):
    _fields_ = [("epochs", u64), ("burnin_epochs", u64), ("contacts", u64),
                ("missed_updates", u64), ("lef_epochs", u64), ("rng_draws", u64),
                ("sort_fallbacks", u64), ("status", u64)]


class EpochRecord(C.Structure):
    _fields_ = [("epoch", u64), ("cell", u64), ("burnin", u64), ("barriers_occupied", u64),
                ("nbarriers", u64), ("num_lefs", u64), ("stalled_rev", u64), ("stalled_fwd", u64),
                ("stalled_both", u64), ("lef_bar", u64), ("lef_lef_primary", u64),
                ("lef_lef_secondary", u64), ("avg_loop_size", C.c_double)]


class BatchTask(C.Structure):
    _fields_ = [("seed", u64), ("target_contacts", u64), ("target_epochs", u64), ("num_lefs", u64),
                ("chrom_id", C.c_int32), ("reserved", u32)]


class ExtraOutputs(C.Structure):
    _fields_ = [("lef_1d_occupancy", C.c_void_p), ("epoch_records", C.c_void_p),
                ("max_epoch_records", u64), ("records_written", C.c_void_p)]


class TraceHeader(C.Structure):
    _fields_ = [("epoch", u64), ("num_active_lefs", u64), ("burnin_completed", u64),
                ("num_burnin_epochs", u64), ("num_contacts", u64), ("rng_draws", u64),
                ("n5prime", u64), ("n3prime", u64), ("digest", u64)]


P64 = C.POINTER(u64)


class TraceRequest(C.Structure):
    _fields_ = [("max_records", u64), ("headers", C.POINTER(TraceHeader)),
                ("rev_pos", P64), ("fwd_pos", P64), ("binding_epoch", P64),
                ("rev_rank", P64), ("fwd_rank", P64), ("rev_move", P64), ("fwd_move", P64),
                ("rev_collision", P64), ("fwd_collision", P64),
                ("max_epochs", u64), ("all_headers", C.POINTER(TraceHeader)),
                ("num_epochs_recorded", u64)]


class PhaseIO(C.Structure):
    _fields_ = [("num_lefs", u64),
                ("rev_pos", P64), ("fwd_pos", P64), ("binding_epoch", P64),
                ("rev_rank", P64), ("fwd_rank", P64), ("rev_move", P64), ("fwd_move", P64),
                ("rev_collision", P64), ("fwd_collision", P64), ("bind_mask", P64),
                ("barrier_state", C.POINTER(C.c_uint8)),
                ("epoch", u64), ("burnin_completed", u32), ("ranks_partially_sorted", u32),
                ("init_ranks", u32), ("adjust_moves", u32), ("prng_state", u64 * 4),
                ("n5prime", u64), ("n3prime", u64), ("lefs_released", u64)]


TRACE_ARRAYS = ("rev_pos", "fwd_pos", "binding_epoch", "rev_rank", "fwd_rank", "rev_move",
                "fwd_move", "rev_collision", "fwd_collision")


def ptr64(arr):
    """Pointer to the data of a contiguous numpy uint64 array (or NULL for None)."""
    if arr is None:
        return None
    assert arr.dtype.itemsize == 8 and arr.flags["C_CONTIGUOUS"]
    return arr.ctypes.data_as(P64)


def make_barriers(barriers):
    """Barrier array from dicts with pos, stp_active, stp_inactive, blocking_dir."""
    arr = (Barrier * max(1, len(barriers)))()
    for i, b in enumerate(barriers):
        arr[i].pos = int(b["pos"])
        arr[i].stp_active = float(b["stp_active"])
        arr[i].stp_inactive = float(b["stp_inactive"])
        arr[i].blocking_dir = int(b["blocking_dir"])
    return arr


class LaunchSetting(C.Structure):
    """mgpu_launch_setting: tuned settings of large batched launches."""
    _fields_ = [("max_lefs", C.c_uint64), ("smem_budget", C.c_uint64), ("carveout_pct", C.c_uint32),
                ("max_cells_per_sm", C.c_uint32)]
