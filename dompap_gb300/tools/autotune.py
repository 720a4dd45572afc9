"""GPU autotuner with the interface of dompap/tools/autotune.py:4-178.

Same procedure as dompap's: time the two neighbour-list build methods (best of
4 forced rebuilds), then scan the skin upward from ``smallest_skin`` in steps
of ``step_skin`` while the time of ``steps`` steps keeps falling (up to half
the smallest box side), and keep the fastest setting. Timings of runs are
device times (CUDA events on the system's stream); builds are timed on the
host around the synchronous rebuild call.

dompap then times its force methods on the system (autotune.py:112-162). On
the GPU every force method is the same neighbour-list step kernel, so the
candidates timed here are that kernel's launch shapes instead: one thread,
four lanes or a warp per particle (the particle's list split over the lanes),
then the resident CTAs per SM it is compiled for (4 or 6); the fastest is set
on the system (``Simulation.set_step_launch``). With ``test_double_loop`` the
step without a list (dompap's "double loop" force method: every pair, one
warp per particle) is timed as well and chosen when it is faster.
"""
from __future__ import annotations

from time import perf_counter


def autotune(sim, steps=100, test_double_loop=True, smallest_skin=0.1, step_skin=0.1, verbose=False,
             plot=False):
    """Return ``sim`` with the fastest neighbour-list method and skin set
    (dompap/tools/autotune.py:4-178; the procedure is the module docstring's)."""
    sim_copy = sim.copy()
    sim_copy.step()
    results = {}
    for method in ("double loop", "cell list"):
        sim_copy.set_neighbor_list(method_str=method)
        times = []
        for _ in range(4):
            tic = perf_counter()
            sim_copy.update_neighbor_list(check=False)
            times.append(perf_counter() - tic)
        results[method] = min(times)
        if verbose:
            print(f"Time to update neighbor list ({method}): {results[method] * 1000:.3f} milliseconds")
    fastest_method = min(results, key=results.get)
    if verbose:
        print(f"Fastest method to update neighbor list: {fastest_method}")
    sim.neighbor_list_method_str = fastest_method
    sim_copy.neighbor_list_method_str = fastest_method

    largest_allowed_skin = min(sim.box_vectors) / 2
    skins, times, updates = [], [], []
    skin = smallest_skin
    old_time = float("inf")
    while skin < largest_allowed_skin:
        before = sim_copy.number_of_neighbor_list_updates
        sim_copy.set_neighbor_list(skin=skin)
        ms = sim_copy.run_timed(steps)
        skins.append(skin)
        times.append(ms / 1000.0)
        updates.append(sim_copy.number_of_neighbor_list_updates - before)
        skin += step_skin
        if ms / 1000.0 > old_time:
            break
        old_time = ms / 1000.0
    if verbose:
        print("Skin | Time per step (ms) | steps/updates")
        for s, t, u in zip(skins, times, updates):
            print(f"{s:4.2f} | {t / steps * 1000:8.5f}          | {steps}/{u}")
    best = skins[times.index(min(times))] if skins else sim.neighbor_list_skin
    if verbose:
        print(f"Optimal parameters: skin={best}")
    sim.set_neighbor_list(skin=best, method_str=fastest_method)

    # launch shape of the step kernel (the GPU's force-method candidates)
    sim_copy.set_neighbor_list(skin=best, method_str=fastest_method)
    n = sim_copy.number_of_particles()
    lane_candidates = [1] + ([4] if n <= 4_000_000 else []) + ([32] if n <= 262_144 else [])
    shape_times = {}

    def time_shape(lanes, blocks):
        sim_copy.set_step_launch(lanes, blocks)
        sim_copy.run(steps)  # graph capture and warm-up
        shape_times[(lanes, blocks)] = min(sim_copy.run_timed(steps) for _ in range(2)) / 1000.0

    for lanes in lane_candidates:
        time_shape(lanes, 0)
    best_lanes = min(shape_times, key=shape_times.get)[0]
    default_blocks = sim_copy.get_step_launch()[1]
    for blocks in (4, 6):
        if blocks != default_blocks:
            time_shape(best_lanes, blocks)
    best_shape = min(shape_times, key=shape_times.get)
    if verbose:
        print("Lanes per particle | CTAs per SM | Time per step (ms)")
        for (lanes, blocks), t in shape_times.items():
            print(f"{lanes:18d} | {blocks if blocks else default_blocks:11d} | {t / steps * 1000:8.5f}")
        print(f"Fastest step launch: {best_shape[0]} lanes per particle, "
              f"{best_shape[1] if best_shape[1] else default_blocks} CTAs per SM")
    sim.set_step_launch(*best_shape)

    # dompap's double-loop force method (autotune.py:112-128): no list, every
    # pair evaluated (one warp per particle); kept when it beats the list step
    method_times = {"neighbor list": shape_times[best_shape]}
    if test_double_loop and n <= 65536:
        sim_copy.set_step_launch(*best_shape)
        sim_copy.force_method_str = "double loop"
        sim_copy.run(steps)
        method_times["double loop"] = min(sim_copy.run_timed(steps) for _ in range(2)) / 1000.0
        sim_copy.force_method_str = "neighbor list"
        if verbose:
            print(f"Time with double loop: {method_times['double loop'] / steps * 1000:0.4f} milliseconds")
    fastest_force = min(method_times, key=method_times.get)
    sim.force_method_str = fastest_force
    if verbose:
        print(f"Fastest method: {sim.force_method_str}")
    sim.__dict__["_autotune_results"] = {"neighbor_list_build_s": results, "skins": skins, "skin_times_s": times,
                                         "step_launch_times_s": shape_times, "step_launch": best_shape,
                                         "force_method_times_s": method_times, "force_method": fastest_force}
    if plot:
        try:
            import matplotlib.pyplot as plt

            plt.plot(skins, times, "o", label="Neighbour list")
            plt.xlabel("Skin")
            plt.ylabel("Time")
            plt.legend()
            plt.show()
        except ImportError:
            pass
    return sim
