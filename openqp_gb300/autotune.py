"""Per-class launch autotuner of the GB300 Fock build.

For every (ab|cd) class the build has a kernel family and three launch
parameters: the family (``FockBuilder.set_kernel_family``: thread per quartet
or warp per quartet, for the classes that have both), the primitive-count
split that sends heavily contracted quartets to the primitive-parallel kernel
(``split_log2``), the quartets a warp takes per work grab (``chunk``), and the
grid cap per SM (``ctas_per_sm``).  The classes run one after another inside a
build and each is bracketed by CUDA events, so one build times every class at
once: the search sets one candidate value for all classes, builds a few times,
and keeps, class by class, the value with the smallest median kernel time; the
family is searched first, then the three parameters one after another
(coordinate search, the others held at their current best).

Results persist in a JSON file keyed by device name, a caller-chosen workload
key, nfocks and precision mode, so a production run tunes once.
"""
import json
import os
import statistics

from .fock import NCLASS

CANDIDATES = {
    "family": [1, 2],
    "split_log2": [6, 7, 8, 9, 10, 64],
    "chunk": [32, 64, 128],
    "ctas_per_sm": [0, 1, 2, 4],
}
# parameters that only the thread-per-quartet kernels use
SMALL_ONLY = ("split_log2", "chunk")


def _device_name():
    import torch
    return torch.cuda.get_device_name(torch.cuda.current_device())


def _class_times(builder, d, reps):
    """Median per-class kernel ms over reps builds (after one untimed build)."""
    build = builder.fock_jk_device
    build(d)
    per = []
    for _ in range(reps):
        build(d)
        per.append(builder.stats()["ms_per_class"])
    return [statistics.median(v[c] for v in per) for c in range(NCLASS)]


def autotune(builder, d, key, cache=None, reps=3, precision="fp64", log=None):
    """Tune builder for density d (torch CUDA float64, (nfocks, ntri)); returns
    the chosen table {"family": [...], "split_log2": [...], "chunk": [...],
    "ctas_per_sm": [...], "class_ms": [...]} and leaves it set on the builder."""
    from .fock import class_labels
    nfocks = d.shape[0] if d.dim() == 2 else 1
    full_key = "%s|%s|nfocks=%d|%s" % (_device_name(), key, nfocks, precision)
    table = None
    if cache and os.path.exists(cache):
        try:
            table = json.load(open(cache)).get(full_key)
        except (OSError, ValueError):
            table = None
    if table is not None:
        builder.set_tuning(table["split_log2"], table["chunk"], table["ctas_per_sm"])
        if "family" in table:
            builder.set_kernel_family(table["family"])
        table = dict(table, cached=True)
        return table
    labels = class_labels()
    family, avail = builder.get_kernel_family()
    best = dict(builder.get_tuning(), family=list(family))

    def apply(t):
        builder.set_tuning(t["split_log2"], t["chunk"], t["ctas_per_sm"])
        builder.set_kernel_family(t["family"])

    base_ms = _class_times(builder, d, reps)
    cur_ms = list(base_ms)
    for name in ("family", "split_log2", "chunk", "ctas_per_sm"):
        trial = {}
        for v in CANDIDATES[name]:
            t = {k: list(vals) for k, vals in best.items()}
            t[name] = [v] * NCLASS
            apply(t)
            trial[v] = _class_times(builder, d, reps)
        for c in range(NCLASS):
            if base_ms[c] == 0.0 or (name == "family" and avail[c] != 3):
                continue
            # the thread-per-quartet parameters of a class that runs warp per quartet
            if name in SMALL_ONLY and (avail[c] == 2 or best["family"][c] == 2):
                continue
            v_best = min(CANDIDATES[name], key=lambda v: trial[v][c])
            if trial[v_best][c] < cur_ms[c]:
                best[name][c] = v_best
                cur_ms[c] = trial[v_best][c]
        if log:
            log("autotune %s: %s" % (name, {labels[c]: best[name][c] for c in range(NCLASS) if base_ms[c] > 0}))
    apply(best)
    table = dict(best, class_ms=_class_times(builder, d, reps), default_class_ms=base_ms)
    if cache:
        try:
            allt = json.load(open(cache)) if os.path.exists(cache) else {}
        except (OSError, ValueError):
            allt = {}
        allt[full_key] = {k: table[k] for k in ("family", "split_log2", "chunk", "ctas_per_sm", "class_ms")}
        os.makedirs(os.path.dirname(os.path.abspath(cache)), exist_ok=True)
        with open(cache, "w") as fh:
            json.dump(allt, fh, indent=1)
    return dict(table, cached=False)


