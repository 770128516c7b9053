"""Benchmark of the GPU BWT path: one step = forward BWT + inverse BWT of the workload's blocks.

Default workload (the single-block configuration): a 64 MiB block of Zipf(1.1) word-token prose (50k-word
vocabulary, 2% random bytes, 200 verbatim 4-64 KiB repeats), seeded synthetic data standing in for the reference's
text corpora. The codec-18 sampling interval for the block (2^23, 7 samples) is used. Other workloads:
markov1 (one 1 MiB order-2 Markov block), degenerate (four 128 MiB blocks: periodic 1 / 7 / 4096 with a flip per
MiB, the Fibonacci word), batch (256 mixed blocks of 16 KiB-16 MiB), slices (the -9 planner's 128 trial slices of
512 KiB) and serve (Poisson compress/decompress requests on the request server).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload prose64|markov1|degenerate|batch|slices|serve]

Output: one JSON line on rank 0.
  value   MiB/s of forward+inverse with the input resident in HBM, timed with CUDA events on the engine's stream,
          L2 flushed (a 256 MiB write) between steps, whole job over all ranks (each rank sorts its own block:
          weak scaling, no collective on the data path);
  e2e     the same metric through the reference-facing C ABI (kolmo_sais_bwt_aux + kolmo_sais_unbwt_aux) with
          pinned host buffers, host<->device copies inside the timed region;
  roofline   the dominant kernel (largest share of device time in a profiled pass of one step, CUDA events around
          every launch of the plain path on the same stream) against the measured HBM copy bandwidth;
  cpu_baseline  the reference's own CPU sorter (compiled on this host from the reference's sources by
          oracle/Makefile) on the whole workload with all host threads, and with one ("t1"); where it is not
          available, the CPU restatement in oracle/ on a bounded sample.
--impl reference times the reference's own CPU sorter (else the restatement) on the same workload, each step the
whole workload, with all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

MIB = 1 << 20
HBM_FALLBACK_GBS = 6800.0


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


# ------------------------------------------------------------------------------------------------ distributed
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def dist_init(world: int, backend: str):
    import torch.distributed as dist

    if world > 1 and not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend)


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def reduce_max(x: float, world: int, device=None) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard(items: list, rank: int, world: int) -> list:
    """Longest-first assignment of independent blocks to ranks (the reference's claim_block order,
    src/core/blocks.c:148-178), returning this rank's share."""
    order = sorted(range(len(items)), key=lambda i: -items[i])
    load = [0] * world
    mine = []
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        load[r] += items[i]
        if r == rank:
            mine.append(i)
    return sorted(mine)


# ------------------------------------------------------------------------------------------------ clocks
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------------ CPU sorter
def cpu_sorter(threads: int | None = None):
    """(kind, fwd(T, r) -> (rc, U, I), inv(U, r, I) -> (rc, T), threads): the reference's own sorter
    (kolmo_sais_bwt_aux / kolmo_sais_unbwt_aux, src/algo/sais/sais.c:12027-12082, compiled on this machine from the
    reference's sources by oracle/Makefile) when it loads here, else the CPU restatement."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    threads = threads or os.cpu_count() or 1
    if O.ref_lib() is not None:
        return ("reference", lambda T, r: O.bwt_aux(T, r, use_ref=True, threads=threads),
                lambda U, r, I: O.unbwt_aux(U, r, I, use_ref=True, threads=threads), threads)
    # the restatement sorts on one thread (SA-IS) and decodes the sampled segments on all threads, like the
    # reference's per-sample decoder
    return ("port", lambda T, r: O.bwt_aux(T, r), lambda U, r, I: O.unbwt_aux(U, r, I, threads=threads), threads)


def time_cpu(T: np.ndarray, r: int, budget_s: float, max_reps: int = 3, threads: int | None = None):
    """fwd+inv MiB/s of the CPU sorter on T (repeated while the time limit budget_s allows)."""
    kind, fwd, inv, threads = cpu_sorter(threads)
    reps, total = 0, 0.0
    while reps < max_reps:
        t0 = time.perf_counter()
        rc, U, I = fwd(T, r)
        rc2, back = inv(U, r, I)
        total += time.perf_counter() - t0
        reps += 1
        assert rc == 0 and rc2 == 0 and np.array_equal(back, T), "CPU sorter failed its round trip"
        if total > budget_s:
            break
    return kind, threads, reps * T.size / MIB / total, reps


def cpu_baseline(blocks: list, budget_s: float = 30.0) -> dict:
    """The CPU sorter on this host: the reference's own sorter on the whole workload with all host threads and with
    one (the reference's -T N and -T 1), else the restatement on a bounded sample of the first block."""
    from kolmo_gb300.host import codec18_rlog

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    nproc = os.cpu_count() or 1
    if O.ref_lib() is not None:
        res = {}
        for t in (nproc, 1):
            tot, nbytes = 0.0, 0
            for T in blocks:
                r = 1 << codec18_rlog(T.size)
                _, _, v, _ = time_cpu(T, r, budget_s=0.0, max_reps=1, threads=t)
                tot += T.size / MIB / v
                nbytes += T.size
            res[t] = nbytes / MIB / tot
        return {"value": round(res[nproc], 2), "unit": "MiB/s", "cores": nproc, "kind": "reference",
                "sample": f"the whole workload ({sum(T.size for T in blocks) / MIB:.0f} MiB), forward+inverse, "
                          f"kolmo_sais_bwt_aux + kolmo_sais_unbwt_aux with threads={nproc}",
                "t1": {"value": round(res[1], 2), "cores": 1}}
    T = blocks[0]
    r = 1 << codec18_rlog(T.size)
    sample = T[: min(T.size, 16 * MIB)]
    kind, threads, v, reps = time_cpu(sample, r, budget_s=12.0)
    return {"value": round(v, 2), "unit": "MiB/s", "cores": threads, "kind": kind,
            "sample": f"first {sample.size / MIB:.0f} MiB of the first block, forward+inverse, {reps} run(s), r={r}; "
                      "forward on one thread, inverse on all"}


# ------------------------------------------------------------------------------------------------ workloads
def prose_block(rank: int, mib: int = 64):
    from kolmo_gb300 import workloads as W

    if rank == 0:
        return W.prose_64mib(mib * MIB)
    return W.zipf_prose(mib * MIB, W.SEED_PROSE_64MIB + rank)


DEGENERATE_KINDS = ("periodic-1", "periodic-7", "periodic-4096", "fibonacci")


def single_blocks(workload: str, rank: int, mib: int):
    """The blocks of a single-block workload (each block is its own forward and inverse call, as the drop-in path
    runs them) and its description."""
    from kolmo_gb300 import workloads as W

    if workload == "markov1":
        return [("markov1", W.markov_1mib())], ("markov1: one 1 MiB order-2 Markov block (64 symbols, Dirichlet 0.3 "
                                                "rows), forward + inverse BWT")
    if workload == "degenerate":
        return ([(k, W.degenerate(k)) for k in DEGENERATE_KINDS],
                "degenerate: four 128 MiB blocks (periodic with periods 1, 7 and 4096 and one random flip per MiB; "
                "the Fibonacci word), each forward + inverse BWT")
    return [("prose64", prose_block(rank, mib))], (f"prose64: one {mib} MiB Zipf(1.1) word-token prose block per GPU, "
                                                   "forward + inverse BWT")


# DRAM bytes per unit (suffix) measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum) on the 16 MiB prose
# case: profiles/traffic_group_thread_lsd_pass_prose16.md (tiny groups) and profiles/lsd_pass_prose16.md (the
# round-0 radix pass, averaged over a 16-pass step). The 64 MiB launch's traffic is scaled by the suffixes it
# processes.
TRAFFIC_PER_SUFFIX = {"group_thread": 35.1, "lsd_pass": 13.9}
RANK_SORTERS = ("tile_sort_rank", "tile_warp_rank", "group_thread", "group_warp", "keygen")


def algorithmic_bytes(rec: dict, round0_launches: int, round0_elems: int) -> float:
    """Algorithmic bytes of one launch, by the doubling model's per-unit figures: round 0 (the sort of every suffix
    by its first W bytes) costs 33 B per suffix in all, credited in equal parts to its radix passes (or, on the tile
    path, to its prefix tile kernels by the suffixes they sort); rank round j costs 48 B per active suffix (read its
    id, gather two ranks, read+write a 12 B (key, id) pair, write SA, rank and compacted id), credited to the kernel
    that sorts the suffix (the large list's suffixes once, at their key generation); the inverse 10 B per byte (psi
    build: read L, write psi; walk: read psi, write text). Scans, segmentation, bucket passes and fixups are
    overhead in the model and get no bytes."""
    k, e = rec["kernel"], rec["elems"]
    if k in RANK_SORTERS:
        return 48.0 * e
    if k == "lsd_pass":
        return 33.0 * round0_elems / max(round0_launches, 1)
    if k in ("tile_sort_prefix", "tile_warp_prefix"):
        return 33.0 * e
    if k in ("inv_walk", "inv_scatter"):
        return 5.0 * e
    return 0.0


def profile_table(prof_f: list, prof_i: list, n: int, h0: int, peak: float) -> tuple:
    """Per-kernel totals with algorithmic bytes, and the per-round table (m_j, h, time, GB/s and fraction of peak)."""
    r0 = [rec for rec in prof_f if rec["round"] == 0 and rec["kernel"] == "lsd_pass"]
    by_kernel = {}
    for rec in prof_f + prof_i:
        d = by_kernel.setdefault(rec["kernel"], {"launches": 0, "ms": 0.0, "bytes": 0.0, "elems": 0})
        d["launches"] += 1
        d["ms"] += rec["ms"]
        d["elems"] += rec["elems"]
        d["bytes"] += algorithmic_bytes(rec, len(r0), n)
    rounds = {}
    for rec in prof_f:
        rr = rounds.setdefault(rec["round"], {"ms": 0.0, "m": 0})
        rr["ms"] += rec["ms"]
        # active suffixes of a rank round: the small, tiny and medium lists (their sort kernels) and the large list
        # (keygen); the keyed tiles sort buckets of the large list and are not counted again
        if rec["kernel"] in RANK_SORTERS:
            rr["m"] += rec["elems"]
    table = []
    for j in sorted(rounds):
        m = rounds[j]["m"] if j > 0 else n
        b = (48.0 if j > 0 else 33.0) * m
        ms = rounds[j]["ms"]
        gbs = b / (ms / 1e3) / 1e9 if ms > 0 else None
        table.append({"round": j, "h": 0 if j == 0 else h0 << (j - 1), "m": m, "ms": round(ms, 4),
                      "GBs": round(gbs, 1) if gbs else None, "frac": round(gbs / peak, 4) if gbs else None})
    return by_kernel, table


def run_ours(args, world, rank, local):
    import torch

    from kolmo_gb300 import codec, native
    from kolmo_gb300.host import codec18_rlog, n_samples

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    named, wname = single_blocks(args.workload, rank, args.block_mib)
    nmax = max(int(T.size) for _, T in named)
    s = torch.cuda.Stream(device=dev)
    eng = codec.Engine()
    eng.config(args.tile_cap, args.tile_ctas, args.msd_ctas, args.small_group, args.warp_path, args.lsd_round0,
               args.lsd_bytes, args.chain_from)
    dT = torch.zeros(nmax + 64, dtype=torch.uint8, device=dev)
    dL = torch.zeros(nmax + 1, dtype=torch.uint8, device=dev)
    dI = torch.zeros(n_samples(nmax, 2), dtype=torch.int32, device=dev)
    dU = torch.zeros(nmax + 64, dtype=torch.uint8, device=dev)
    dOut = torch.zeros(nmax + 64, dtype=torch.uint8, device=dev)
    # the text of every block stays resident; a step copies none of it from the host
    resident = [torch.from_numpy(T).to(dev) for _, T in named]
    flush = torch.empty(256 * MIB, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    total = sum(int(T.size) for _, T in named)

    def load(b):
        """puts block b's resident text into the engine's input buffer (outside the timed region)"""
        n = int(named[b][1].size)
        with torch.cuda.stream(s):
            dT[:n].copy_(resident[b])
            dT[n:n + 64].zero_()

    def one_block(b, plain=False):
        """forward + inverse of block b (already in dT); returns (fwd ms, inv ms) from CUDA events on the engine
        stream."""
        T = named[b][1]
        n = int(T.size)
        r = 1 << codec18_rlog(n)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        ev[0].record(s)
        rc = eng.fwd(dT, dL, dI, [(0, n, r, 0)], stream=s, plain=plain)
        ev[1].record(s)
        rc2 = eng.wait()[0]
        if rc or rc2:
            raise RuntimeError(f"forward failed: {rc} {rc2} {native.last_error()}")
        p0 = int(dI[0].item())
        ev[2].record(s)
        with torch.cuda.stream(s):
            dU[:p0].copy_(dL[:p0])
            dU[p0:n].copy_(dL[p0 + 1:n + 1])
        rc = eng.inv(dU, dOut, [(0, n, p0)], stream=s, plain=plain)
        ev[3].record(s)
        rc2, st = eng.wait(1)
        if rc or rc2:
            raise RuntimeError(f"inverse failed: {rc} {rc2} {native.last_error()}")
        s.synchronize()
        return ev[0].elapsed_time(ev[1]), ev[2].elapsed_time(ev[3])

    # warm-up (also the correctness check of this run)
    load(0)
    for _ in range(max(args.warmup, 1)):
        for b in range(len(named)):
            if len(named) > 1:
                load(b)
            one_block(b, plain=args.plain)
            assert torch.equal(dOut[:named[b][1].size], resident[b]), f"round trip failed: {named[b][0]}"

    clocks = Clocks(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    times, tf, ti = [], [], []
    per_block = [[0.0, 0.0] for _ in named]
    for _ in range(args.steps):
        step = 0.0
        for b in range(len(named)):
            if len(named) > 1:
                load(b)
            with torch.cuda.stream(s):
                flush.fill_(1)
            f_ms, i_ms = one_block(b, plain=args.plain)
            tf.append(f_ms)
            ti.append(i_ms)
            per_block[b][0] += f_ms
            per_block[b][1] += i_ms
            step += f_ms + i_ms
        times.append(step)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(world)
    total_ms = reduce_max(sum(times), world, dev)
    value = world * args.steps * total / MIB / (total_ms / 1e3)
    if args.skip_extras:  # timed steps only (profiler runs)
        return {"metric": "bwt_fwd_inv_MiB_per_s", "value": round(value, 2), "unit": "MiB/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3),
                "fwd_ms": round(sum(tf) / args.steps, 3), "inv_ms": round(sum(ti) / args.steps, 3),
                "bytes": total, "skip_extras": True,
                "cfg": [args.tile_cap, args.tile_ctas, args.msd_ctas, args.small_group, args.warp_path,
                        args.lsd_round0, args.lsd_bytes]}

    # profiled pass (plain path, CUDA events around every launch on stream s), one per block
    peak, peak_kind = peaks()
    by_kernel, blocks_out = {}, []
    launches = 0
    for b, (name, T) in enumerate(named):
        n = int(T.size)
        r = 1 << codec18_rlog(n)
        load(b)
        eng.profile(True)
        assert eng.fwd(dT, dL, dI, [(0, n, r, 0)], stream=s, plain=True) == 0 and eng.wait()[0] == 0
        prof_f = eng.profile_read()
        p0 = int(dI[0].item())
        with torch.cuda.stream(s):
            dU[:p0].copy_(dL[:p0])
            dU[p0:n].copy_(dL[p0 + 1:n + 1])
        assert eng.inv(dU, dOut, [(0, n, p0)], stream=s, plain=True) == 0 and eng.wait(1)[0] == 0
        prof_i = eng.profile_read()
        eng.profile(False)
        if args.profile_out and rank == 0:
            with open(args.profile_out if len(named) == 1 else f"{args.profile_out}.{name}", "w") as f:
                json.dump({"forward": prof_f, "inverse": prof_i}, f)
        launches += len(prof_f) + len(prof_i)
        lc = eng.last_config()
        h0 = lc["lsd_bytes"] if lc["lsd_round0"] else 8  # prefix bytes round 0 sorts (the first rank round's h)
        bk, table = profile_table(prof_f, prof_i, n, h0, peak)
        for k, d in bk.items():
            a = by_kernel.setdefault(k, {"launches": 0, "ms": 0.0, "bytes": 0.0, "elems": 0})
            for f in a:
                a[f] += d[f]
        blocks_out.append({"block": name, "bytes": n, "r": r, "fwd_ms": round(per_block[b][0] / args.steps, 3),
                           "inv_ms": round(per_block[b][1] / args.steps, 3), "rounds": table})
    tot_ms = sum(d["ms"] for d in by_kernel.values())
    dom = max((k for k in by_kernel if k != "control"), key=lambda k: by_kernel[k]["ms"])
    dd = by_kernel[dom]
    achieved = dd["bytes"] / (dd["ms"] / 1e3) / 1e9 if dd["ms"] > 0 else 0.0

    # e2e through the drop-in C ABI with pinned host buffers
    e2e = run_e2e([T for _, T in named], args.steps, max(args.warmup, 1), world, dev)

    cfg = {"workload": wname, "bytes": total, "blocks": [{"block": nm, "bytes": int(T.size),
                                                          "r": 1 << codec18_rlog(int(T.size))} for nm, T in named],
           "l2": "flushed before every block (256 MiB write)", "parallelism": f"replicas{world}", "tile_cap": 4096}
    out = {
        "metric": "bwt_fwd_inv_MiB_per_s", "value": round(value, 2), "unit": "MiB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": cfg,
        "fwd_MiB_per_s": round(args.steps * total / MIB / (sum(tf) / 1e3), 2),
        "inv_MiB_per_s": round(args.steps * total / MIB / (sum(ti) / 1e3), 2),
        "e2e": e2e,
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "peak_source": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": None,
                     "launches_per_step": dd["launches"], "share": round(dd["ms"] / tot_ms, 4),
                     "bytes_model": "doubling model: round 0 33 B per suffix over its radix passes, rank round 48 B "
                                    "per active suffix, inverse 10 B per byte; scans, segmentation, bucket passes "
                                    "and fixups get none"},
        "kernel_shares": {k: round(v["ms"] / tot_ms, 4) for k, v in sorted(by_kernel.items(), key=lambda x: -x[1]["ms"])},
        "gpu_launches": args.steps * launches,
        "clocks": clk,
    }
    if len(blocks_out) == 1:
        out["rounds"] = blocks_out[0]["rounds"]
    else:
        out["blocks"] = blocks_out
    if dom == "lsd_pass":
        # the pass itself: every pass reads and writes each suffix's 8-byte item (id and one 4-byte key group)
        item = 16.0 * dd["elems"] / (dd["ms"] / 1e3) / 1e9
        out["roofline"]["item_traffic"] = {"achieved": round(item, 1), "frac": round(item / peak, 4),
                                           "model": "16 B per suffix per radix pass (read and write its item)"}
    if dom in TRAFFIC_PER_SUFFIX:
        elems = dd["elems"] / max(dd["launches"], 1)
        out["roofline"]["traffic"] = round(TRAFFIC_PER_SUFFIX[dom] * elems)
        out["roofline"]["traffic_source"] = "ncu dram bytes per suffix on the 16 MiB case x suffixes per launch"
    if rank == 0:
        out["cpu_baseline"] = cpu_baseline([T for _, T in named])
    return out


SLICE_BYTES, SLICE_COUNT = 512 << 10, 128


def batch_blocks(workload: str):
    """The blocks of a batch workload and its description: the mixed batch (256 blocks of 16 KiB-16 MiB,
    log-uniform; order-2 Markov, ACGT with 0.1% N, templated log lines), or the -9 slice trials (128 consecutive
    512 KiB slices of the 64 MiB prose block, each sorted on its own, as the level-9 planner sorts trial slices of a
    file: src/core/blocks.c:399-517)."""
    from kolmo_gb300 import workloads as W

    if workload == "slices":
        T = W.prose_64mib()
        texts = [T[i * SLICE_BYTES:(i + 1) * SLICE_BYTES] for i in range(SLICE_COUNT)]
        return texts, (f"slices{SLICE_COUNT}: {SLICE_COUNT} consecutive {SLICE_BYTES >> 10} KiB slices of the 64 MiB "
                       "prose block (the -9 slice trials), forward + inverse BWT, one graph launch per direction")
    return [t for _, t in W.mixed_batch()], ("batch256: 256 blocks, log-uniform 16 KiB-16 MiB (order-2 Markov, "
                                             "ACGT, log lines), forward + inverse BWT, one graph launch per direction")


def run_batch(args, world, rank, local):
    """A batch workload (batch_blocks): one step = forward + inverse of every block. Timed three ways: the batched
    graph path (one engine call per direction for the whole batch, device-resident buffers), the plain per-block path
    (one call per block, host-driven rounds), and e2e through the batch C ABI (kgbwt_fwd_batch / kgbwt_inv_batch,
    host buffers). Each rank takes a longest-first share of the blocks (weak scaling by blocks, no collective)."""
    import torch

    from kolmo_gb300 import codec, native
    from kolmo_gb300 import workloads as W
    from kolmo_gb300.host import codec18_rlog, n_samples

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    allb, wname = batch_blocks(args.workload)
    mine = shard([int(t.size) for t in allb], rank, world)
    texts = [np.ascontiguousarray(allb[i]) for i in mine]
    offs, o = [], 0
    for t in texts:
        offs.append(o)
        o += (t.size + 15) // 16 * 16
    total = sum(int(t.size) for t in texts)
    rs = [1 << codec18_rlog(int(t.size)) for t in texts]
    iouts, k = [], 0
    for t, r in zip(texts, rs):
        iouts.append(k)
        k += n_samples(int(t.size), r)
    hbuf = np.zeros(o + 64, np.uint8)
    for t, off in zip(texts, offs):
        hbuf[off:off + t.size] = t
    dT = torch.from_numpy(hbuf).to(dev)
    dL = torch.zeros(o + len(texts) + 64, dtype=torch.uint8, device=dev)
    dI = torch.zeros(k, dtype=torch.int32, device=dev)
    dU = torch.zeros_like(dT)
    dOut = torch.zeros_like(dT)
    flush = torch.empty(256 * MIB, dtype=torch.uint8, device=dev)
    s = torch.cuda.Stream(device=dev)
    eng = codec.Engine()
    eng.config(args.tile_cap, args.tile_ctas, args.msd_ctas, args.small_group, args.warp_path, args.lsd_round0,
               args.lsd_bytes, args.chain_from)
    fblocks = [(off, int(t.size), r, io) for t, off, r, io in zip(texts, offs, rs, iouts)]

    def to_u(b_list, I):
        with torch.cuda.stream(s):
            for (off, n, r, io), bi in b_list:
                p0 = int(I[io])
                dU[off:off + p0].copy_(dL[off + bi:off + bi + p0])
                dU[off + p0:off + n].copy_(dL[off + bi + p0 + 1:off + bi + n + 1])

    def step_batched():
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record(s)
        if eng.fwd(dT, dL, dI, fblocks, stream=s) or eng.wait()[0]:
            raise RuntimeError(f"batched forward failed: {native.last_error()}")
        I = dI.cpu().numpy()
        to_u([(fb, b) for b, fb in enumerate(fblocks)], I)
        iblocks = [(off, n, int(I[io])) for off, n, r, io in fblocks]
        if eng.inv(dU, dOut, iblocks, stream=s) or eng.wait(len(iblocks))[0]:
            raise RuntimeError(f"batched inverse failed: {native.last_error()}")
        ev[1].record(s)
        return ev

    def step_plain():
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record(s)
        for b, (off, n, r, io) in enumerate(fblocks):
            # one block per call, laid out as a batch of one at the block's own offset
            if eng.fwd(dT[off:], dL[off + b:], dI[io:], [(0, n, r, 0)], stream=s, plain=True) or eng.wait()[0]:
                raise RuntimeError(f"plain forward failed: {native.last_error()}")
            p0 = int(dI[io].item())
            with torch.cuda.stream(s):
                dU[off:off + p0].copy_(dL[off + b:off + b + p0])
                dU[off + p0:off + n].copy_(dL[off + b + p0 + 1:off + b + n + 1])
            if eng.inv(dU[off:], dOut[off:], [(0, n, p0)], stream=s, plain=True) or eng.wait(1)[0]:
                raise RuntimeError(f"plain inverse failed: {native.last_error()}")
        ev[1].record(s)
        return ev

    for _ in range(max(args.warmup, 1)):
        step_batched()
    s.synchronize()
    for t, off in zip(texts, offs):
        assert torch.equal(dOut[off:off + t.size].cpu(), torch.from_numpy(t)), "batched round trip failed"
    clocks = Clocks(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    tb = 0.0
    for _ in range(args.steps):
        with torch.cuda.stream(s):
            flush.fill_(1)
        ev = step_batched()
        s.synchronize()
        tb += ev[0].elapsed_time(ev[1])
    clk = clocks.stop()
    barrier(world)
    tb = reduce_max(tb, world, dev)
    value = world * args.steps * total / MIB / (tb / 1e3)
    # the plain per-block path: one untimed pass, then one timed pass
    dOut.zero_()
    step_plain()
    s.synchronize()
    ev = step_plain()
    s.synchronize()
    tp = reduce_max(ev[0].elapsed_time(ev[1]), world, dev)
    for t, off in zip(texts, offs):
        assert torch.equal(dOut[off:off + t.size].cpu(), torch.from_numpy(t)), "plain round trip failed"
    plain_v = world * total / MIB / (tp / 1e3)
    ws = eng.workspace_bytes()
    eng.close()  # the C ABI below sorts on the library's own engine: release this one's workspace first
    del dT, dL, dI, dU, dOut, flush
    torch.cuda.empty_cache()
    # e2e: the batch C ABI with host buffers
    jobs = [(t, r) for t, r in zip(texts, rs)]
    rc, outs = codec.fwd_batch(jobs)
    assert rc == 0 and all(o_[0] == 0 for o_ in outs)
    ijobs = [(U, r, I) for (_, U, I), r in zip(outs, rs)]
    barrier(world)
    te = 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        rc, outs = codec.fwd_batch(jobs)
        rc2, backs = codec.inv_batch([(U, r, I) for (_, U, I), r in zip(outs, rs)])
        te += time.perf_counter() - t0
        assert rc == 0 and rc2 == 0
    for (rcb, back), t in zip(backs, texts):
        assert rcb == 0 and np.array_equal(back, t), "C ABI batch round trip failed"
    te = reduce_max(te, world, dev)
    e2e_v = world * args.steps * total / MIB / te
    out = {
        "metric": "bwt_fwd_inv_MiB_per_s", "value": round(value, 2), "unit": "MiB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(tb / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": wname,
                   "blocks": len(texts), "bytes": total, "l2": "flushed between steps (256 MiB write)",
                   "parallelism": f"blocks sharded longest-first over {world} rank(s)"},
        "plain_per_block_MiB_per_s": round(plain_v, 2),
        "batched_over_plain": round(value / plain_v, 2),
        "e2e": {"value": round(e2e_v, 2), "unit": "MiB/s", "h2d_bytes_per_step": 2 * total,
                "d2h_bytes_per_step": 2 * total + 4 * k, "path": "kgbwt_fwd_batch + kgbwt_inv_batch, host buffers"},
        "workspace_bytes": ws,
        "clocks": clk,
    }
    return out


def run_serve(args, world, rank, local):
    """The serving workload: Poisson arrivals (rate --rate per second) of compress (30%, forward BWT) and decompress
    (70%, inverse BWT) requests, lognormal sizes (median 256 KiB, sigma 1.5, capped at 128 MiB) from the three batch
    sources, on the request server (--slots workers, 150 GB HBM budget, host buffers in and out). Reports p50/p99
    latency (submission to completion) and MiB/s (request bytes over first arrival to last completion), next to the
    serial per-request plain path on the same arrivals (each request's plain-path service time measured alone, then
    a FIFO single server replayed over the arrival times). Each rank serves its own stream (weak scaling)."""
    import threading

    import torch

    from kolmo_gb300 import codec, native
    from kolmo_gb300 import workloads as W
    from kolmo_gb300.host import codec18_rlog

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    count = args.requests
    sizes, gaps, mix, src = W.requests(W.SEED_SERVE + rank, count, rate=args.rate)
    reqs = []
    for i in range(count):
        n = max(int(sizes[i]), 2)
        T = W.source_block(int(src[i]), n, W.SEED_SERVE * 7 + i)
        r = 1 << codec18_rlog(n)
        reqs.append(("fwd" if mix[i] < 300 else "inv", T, r))
    # decompress payloads: the BWT of each decompress request (made before the timed region)
    payload = []
    for kind, T, r in reqs:
        if kind == "inv":
            rc, U, I = codec.bwt_aux(T, r)
            assert rc == 0
            payload.append((U, I))
        else:
            payload.append(None)
    arrivals = np.cumsum(gaps) - gaps[0]
    total = sum(int(T.size) for _, T, _ in reqs)

    # one server for the warm-up rounds and the timed round: its workers keep their workspaces resident, as a
    # long-running server does
    srv = codec.Server(slots=args.slots, hbm_budget=150 * 10**9)

    def serve_once():
        before = srv.stats()
        handles = [None] * count
        t0 = time.perf_counter()

        def submitter():
            for i, (kind, T, r) in enumerate(reqs):
                d = t0 + arrivals[i] - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                handles[i] = srv.submit_fwd(T, r) if kind == "fwd" else srv.submit_inv(payload[i][0], r, payload[i][1])

        th = threading.Thread(target=submitter)
        th.start()
        th.join()
        lat = np.zeros(count)
        for i, h in enumerate(handles):
            st, rc, us = srv.wait(h[0], 600000)
            if st != 1 or rc != 0:
                raise RuntimeError(f"request {i} failed: {st} {rc} {native.last_error()}")
            lat[i] = us / 1e3
        t_end = time.perf_counter()
        stats = srv.stats()
        stats = {"batches": stats["batches"] - before["batches"], "hbm_peak": stats["hbm_peak"]}
        # results equal the drop-in calls (spot check every 8th request)
        for i in range(0, count, 8):
            kind, T, r = reqs[i]
            if kind == "fwd":
                rc, U, I = codec.bwt_aux(T, r)
                assert np.array_equal(handles[i][1], U) and np.array_equal(handles[i][2], I)
            else:
                assert np.array_equal(handles[i][1], T)
        return lat, t_end - t0, stats

    for _ in range(max(args.warmup, 1) if args.warmup else 1):
        serve_once()
    barrier(world)
    lat, wall, stats = serve_once()
    srv.close()
    value = total / MIB / wall
    # serial per-request plain path: service times alone, then a FIFO single server over the same arrivals
    svc = np.zeros(count)
    for i, (kind, T, r) in enumerate(reqs):
        t1 = time.perf_counter()
        if kind == "fwd":
            rc, outs = codec.fwd_batch([(T, r)], plain=True)
        else:
            rc, outs = codec.inv_batch([(payload[i][0], r, payload[i][1])], plain=True)
        svc[i] = time.perf_counter() - t1
        assert rc == 0
    fin = 0.0
    slat = np.zeros(count)
    for i in range(count):
        start = max(arrivals[i], fin)
        fin = start + svc[i]
        slat[i] = (fin - arrivals[i]) * 1e3
    serial_v = total / MIB / fin
    value = reduce_max(-value, world, dev) * -1.0 if world > 1 else value
    return {
        "metric": "serve_MiB_per_s", "value": round(world * value, 2), "unit": "MiB/s", "n_gpus": world,
        "steps": 1, "warmup": args.warmup, "ms_per_step": round(wall * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": f"serve: {count} Poisson requests at {args.rate}/s, 30% compress / 70% decompress, "
                               "lognormal sizes (median 256 KiB, sigma 1.5, cap 128 MiB), batch sources",
                   "slots": args.slots, "hbm_budget": 150 * 10**9, "bytes": total,
                   "server": "warm: the warm-up rounds run the same stream on the same server"},
        "p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
        "serial_plain": {"value": round(serial_v, 2), "unit": "MiB/s",
                         "p50_ms": round(float(np.percentile(slat, 50)), 3),
                         "p99_ms": round(float(np.percentile(slat, 99)), 3)},
        "server": {"batches": stats["batches"], "hbm_peak": stats["hbm_peak"]},
    }


def run_e2e(texts: list, steps: int, warmup: int, world: int, dev):
    """The workload through the drop-in C ABI (kolmo_sais_bwt_aux, then kolmo_sais_unbwt_aux on its output) from
    pinned host buffers; every step copies each block's text in and its BWT and decoded text out."""
    import torch

    from kolmo_gb300 import native
    from kolmo_gb300.host import codec18_rlog, n_samples

    L = native.lib()
    A = np.zeros(1, np.int32)
    bufs = []
    for T in texts:
        n = int(T.size)
        r = 1 << codec18_rlog(n)
        Th = torch.from_numpy(T.copy()).pin_memory()
        Uh = torch.empty(n, dtype=torch.uint8).pin_memory()
        Bh = torch.empty(n, dtype=torch.uint8).pin_memory()
        bufs.append((n, r, Th, Uh, Bh, np.zeros(n_samples(n, r), np.int32)))

    def one():
        for n, r, Th, Uh, Bh, I in bufs:
            rc = L.kolmo_sais_bwt_aux(Th.data_ptr(), Uh.data_ptr(), A.ctypes.data, n, r, I.ctypes.data, 1)
            rc2 = L.kolmo_sais_unbwt_aux(Uh.data_ptr(), Bh.data_ptr(), A.ctypes.data, n, r, I.ctypes.data, 1)
            if rc or rc2:
                raise RuntimeError(f"C ABI round trip failed: {rc} {rc2} {native.last_error()}")

    for _ in range(warmup):
        one()
    for n, r, Th, Uh, Bh, I in bufs:
        assert torch.equal(Bh, Th), "C ABI round trip differs"
    barrier(world)
    t = 0.0
    for _ in range(steps):
        t0 = time.perf_counter()
        one()
        t += time.perf_counter() - t0
    t = reduce_max(t, world, dev)
    total = sum(b[0] for b in bufs)
    return {"value": round(world * steps * total / MIB / t, 2), "unit": "MiB/s", "h2d_bytes_per_step": 2 * total,
            "d2h_bytes_per_step": 2 * total + sum(4 * int(b[5].size) for b in bufs),
            "path": "kolmo_sais_bwt_aux + kolmo_sais_unbwt_aux, pinned host buffers"}


def run_reference(args, world, rank):
    """The reference's own CPU sorter on the same workload, on this host's cores: kolmo_sais_bwt_aux and
    kolmo_sais_unbwt_aux compiled from the reference's sources (oracle/Makefile) with every host thread, each step the
    whole workload. Where that library is not available the CPU restatement runs on a bounded sample instead."""
    if rank != 0:
        return None
    from kolmo_gb300.host import codec18_rlog

    named, wname = single_blocks(args.workload if args.workload in ("markov1", "degenerate") else "prose64", 0,
                                 args.block_mib)
    texts = [T for _, T in named]
    kind, fwd, inv, threads = cpu_sorter()
    if kind == "reference":
        samples = texts
        desc = (f"the whole workload ({sum(T.size for T in texts) / MIB:.0f} MiB) per step, forward+inverse, "
                f"kolmo_sais_bwt_aux + kolmo_sais_unbwt_aux with threads={threads}")
    else:
        # size the per-step sample so that warm-up + steps stay within about two minutes
        T = texts[0]
        r = 1 << codec18_rlog(T.size)
        probe = T[: 4 * MIB]
        t0 = time.perf_counter()
        rc, U, I = fwd(probe, r)
        inv(U, r, I)
        speed = probe.size / (time.perf_counter() - t0)  # bytes/s
        per_step = 120.0 / max(args.steps + args.warmup, 1)
        samples = [T[: int(min(T.size, max(4 * MIB, speed * per_step)))]]
        desc = (f"first {samples[0].size / MIB:.1f} MiB of the first block per step, forward+inverse, r={r}; "
                f"forward on one thread (SA-IS restatement), inverse on {threads} threads (per-sample decode)")
    rs = [1 << codec18_rlog(S.size) for S in samples]
    for _ in range(args.warmup):
        for S, r in zip(samples, rs):
            fwd(S, r)
    t = 0.0
    for _ in range(args.steps):
        for S, r in zip(samples, rs):
            t0 = time.perf_counter()
            rc, U, I = fwd(S, r)
            rc2, back = inv(U, r, I)
            t += time.perf_counter() - t0
            assert rc == 0 and rc2 == 0
    total = sum(S.size for S in samples)
    v = args.steps * total / MIB / t
    return {"metric": "bwt_fwd_inv_MiB_per_s", "value": round(v, 2), "unit": "MiB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t / args.steps * 1e3, 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": wname, "bytes": int(sum(T.size for T in texts)),
                       "blocks": [{"block": nm, "bytes": int(T.size), "r": 1 << codec18_rlog(int(T.size))}
                                  for nm, T in named], "parallelism": "cpu", "same_config": kind == "reference"},
            "cpu_baseline": {"value": round(v, 2), "unit": "MiB/s", "cores": threads, "kind": kind, "sample": desc},
            "e2e": {"value": round(v, 2), "unit": "MiB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def probe_random():
    """Random 4-byte access rates of this GPU against the size of the array they hit: 64 M independent gathers
    (torch index_select with int32 indices) and scatters (index_copy_ with int64 indices), CUDA events, best of four.
    The rates include each call's sequential index read and, for gathers, its output write. They are the ceiling of a
    kernel whose loads are random and independent: the inverse walk's psi loads and the rank rounds' rank gathers
    hit arrays of 4 bytes per text byte (256 MiB for a 64 MiB block)."""
    import torch

    nops = 64 << 20
    g = torch.Generator(device="cuda")
    out = []
    for mib in (64, 128, 256, 1024, 4096):
        n = (mib << 20) // 4
        arr = torch.ones(n, dtype=torch.int32, device="cuda")
        g.manual_seed(mib)
        idx = torch.randint(0, n, (nops,), device="cuda", dtype=torch.int64, generator=g)
        idx32 = idx.to(torch.int32)
        src = torch.zeros(nops, dtype=torch.int32, device="cuda")

        def best(fn):
            t = []
            for _ in range(5):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                fn()
                e1.record()
                torch.cuda.synchronize()
                t.append(e0.elapsed_time(e1))
            return min(t[1:])
        tg = best(lambda: torch.index_select(arr, 0, idx32))
        ts = best(lambda: arr.index_copy_(0, idx, src))
        out.append({"array_mib": mib, "gathers_G_per_s": round(nops / tg / 1e6, 1),
                    "scatters_G_per_s": round(nops / ts / 1e6, 1)})
        del arr, idx, idx32, src
    return {"probe": "random_4byte_access", "ops": nops, "device": torch.cuda.get_device_name(), "results": out}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="prose64",
                    choices=["prose64", "markov1", "degenerate", "batch", "slices", "serve"])
    ap.add_argument("--rate", type=float, default=1000.0, help="serve: Poisson arrival rate (requests per second)")
    ap.add_argument("--requests", type=int, default=400, help="serve: requests in the stream")
    ap.add_argument("--slots", type=int, default=3, help="serve: server workers")
    ap.add_argument("--block-mib", type=int, default=64, help="block size (the benchmark configuration is 64)")
    ap.add_argument("--tile-cap", type=int, default=0, help="engine tile capacity (4096 or 8192; 0 = default)")
    ap.add_argument("--tile-ctas", type=int, default=0)
    ap.add_argument("--msd-ctas", type=int, default=0)
    ap.add_argument("--small-group", type=int, default=-1)
    ap.add_argument("--warp-path", type=int, default=-1)
    ap.add_argument("--lsd-round0", type=int, default=-1)
    ap.add_argument("--lsd-bytes", type=int, default=-1, help="prefix bytes of the LSD round 0 (8, 12 or 16)")
    ap.add_argument("--chain-from", type=int, default=-1, help="first rank round with repeat chains (0: none)")
    ap.add_argument("--profile-out", default="", help="write the per-launch profile of the profiled step here")
    ap.add_argument("--plain", action="store_true",
                    help="time the plain path (one launch per kernel, host sync per round) instead of the graph")
    ap.add_argument("--skip-extras", action="store_true",
                    help="timed steps only: no e2e, profiled pass or CPU baseline (for profiler captures)")
    ap.add_argument("--probe-random", action="store_true",
                    help="print this GPU's random 4-byte gather and scatter rates by array size, and exit")
    args = ap.parse_args()
    if args.probe_random:
        print(json.dumps(probe_random()), flush=True)
        return
    world, rank, local = dist_env()
    if args.impl == "reference":
        out = run_reference(args, world, rank)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    import torch

    dist_init(world, "nccl" if torch.cuda.is_available() else "gloo")
    if args.workload in ("batch", "slices"):
        out = run_batch(args, world, rank, local)
    elif args.workload == "serve":
        out = run_serve(args, world, rank, local)
    else:
        out = run_ours(args, world, rank, local)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
