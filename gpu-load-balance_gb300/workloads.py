"""Seeded synthetic workloads of the benchmark configurations (shared by bench.py and the
tests). Every draw comes from the same counter-based hash as the particle generators, so a
workload is reproducible from its seed alone.

  batched (128 instances): particle counts log-uniform in [2^14, 2^22], leaf counts 2^k with
      k uniform in {6..12}, alternately uniform and Plummer-clustered particles.
  served: Poisson arrivals (exponential gaps at a given rate) mixing new instances (sizes as
      the batched workload) and rebalances (Gaussian displacement) of resident instances.
"""
from __future__ import annotations

from dataclasses import dataclass

M64 = (1 << 64) - 1


def mix64(z: int) -> int:
    z = (z + 0x9E3779B97F4A7C15) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def draw(seed: int, counter: int) -> int:
    """The generators' counter-based draw: mix64(mix64(seed) + counter * K)."""
    return mix64((mix64(seed & M64) + counter * 0xD1B54A32D192ED03) & M64)


def unit(seed: int, counter: int) -> float:
    return (draw(seed, counter) >> 11) * 2.0 ** -53


@dataclass
class InstanceSpec:
    kind: str       # "uniform" | "plummer"
    seed: int
    n: int
    d: int


def batched_instances(seed: int, count: int = 128, lo_log2: int = 14, hi_log2: int = 22,
                      leaf_log2=(6, 12)) -> list[InstanceSpec]:
    out = []
    for i in range(count):
        n = int(2.0 ** (lo_log2 + (hi_log2 - lo_log2) * unit(seed, 3 * i)))
        k = leaf_log2[0] + draw(seed, 3 * i + 1) % (leaf_log2[1] - leaf_log2[0] + 1)
        out.append(InstanceSpec("uniform" if i % 2 == 0 else "plummer",
                                draw(seed ^ 0xBA7C4ED, i), n, 1 << k))
    return out


@dataclass
class Request:
    t: float            # arrival time (s)
    kind: str           # "build" | "rebalance"
    spec: InstanceSpec | None   # build: the new instance
    target: int         # rebalance: index of an earlier build request
    seed: int           # rebalance: displacement seed


def served_stream(seed: int, rate: float, count: int, rebalance_frac: float = 0.5,
                  sizes=(14, 20)) -> list[Request]:
    """Poisson request stream: exponential inter-arrival times at `rate` per second; each
    request is a rebalance of a random earlier build with probability rebalance_frac."""
    import math
    out, t, builds = [], 0.0, []
    specs = batched_instances(seed ^ 0x5E7E, count, sizes[0], sizes[1])
    for i in range(count):
        t += -math.log(1.0 - unit(seed, 4 * i)) / rate
        if builds and unit(seed, 4 * i + 1) < rebalance_frac:
            tgt = builds[draw(seed, 4 * i + 2) % len(builds)]
            out.append(Request(t, "rebalance", None, tgt, draw(seed, 4 * i + 3)))
        else:
            builds.append(i)
            out.append(Request(t, "build", specs[i], -1, 0))
    return out
