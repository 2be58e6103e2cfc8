"""Generate the golden fixtures from the reference itself.

Run where the reference tree exists (it builds oracle/_ref/libvsmcref.so from
the reference's own sources with `make -C oracle ref`):

    python tests/golden/make_golden.py

Every array comes from the reference's code (CounterEngine, u01, the
distributions, U01Sequence*, the Resample* functors and transforms, Weight,
Sampler<T> runs); inputs are seeded numpy draws stored beside the outputs.
The fixtures are small and committed; tests/test_oracle_golden.py checks the
C restatement against them on any host.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import binding  # noqa: E402

P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731

KEYS32 = np.array([[0, 0], [0x12345678, 0x9ABCDEF0], [0xFFFFFFFF, 0xFFFFFFFF]],
                  np.uint32)
CTRS32 = np.array([[0, 0, 0, 0], [0xFFFFFFFF - 300, 0, 0, 0],
                   [0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFE],
                   [0xFFFFFFFF] * 4, [7, 3, 2, 1]], np.uint32)
KEYS64 = np.array([[0, 0, 0, 0], [0x0123456789ABCDEF, 0, 2**64 - 1, 42]],
                  np.uint64)
CTRS64 = np.array([[0, 0, 0, 0], [2**64 - 300, 0, 0, 0],
                   [2**64 - 1, 2**64 - 1, 5, 0]], np.uint64)
NWORDS = 2053


def rng_words(R):
    out = {}
    for b in (0, 1):
        a = np.zeros((len(KEYS32), len(CTRS32), NWORDS), np.uint32)
        for i, k in enumerate(KEYS32):
            for j, c in enumerate(CTRS32):
                R.ref_philox4x32_words(P(np.ascontiguousarray(k)),
                                       P(np.ascontiguousarray(c)), NWORDS,
                                       P(a[i, j]), b)
        out[f"philox_bulk{b}"] = a
        a = np.zeros((len(KEYS64), len(CTRS64), NWORDS), np.uint64)
        for i, k in enumerate(KEYS64):
            for j, c in enumerate(CTRS64):
                R.ref_threefry4x64_words(P(np.ascontiguousarray(k)),
                                         P(np.ascontiguousarray(c)), NWORDS,
                                         P(a[i, j]), b)
        out[f"threefry_bulk{b}"] = a
    out.update(keys32=KEYS32, ctrs32=CTRS32, keys64=KEYS64, ctrs64=CTRS64)
    return out


def u01(R, rng):
    u32 = rng.integers(0, 2**32, 4096, dtype=np.uint64).astype(np.uint32)
    u32[:4] = [0, 1, 0xFFFFFFFF, 0xFFFFFFFE]
    u64 = rng.integers(0, 2**64 - 1, 4096, dtype=np.uint64, endpoint=True)
    u64[:3] = [0, 1, 2**64 - 1]
    out = {"u32": u32, "u64": u64}
    for lr in range(4):
        a = np.zeros(len(u32))
        R.ref_u01_u32_f64(lr, len(u32), P(u32), P(a))
        out[f"u32_f64_{lr}"] = a
        f = np.zeros(len(u32), np.float32)
        R.ref_u01_u32_f32(lr, len(u32), P(u32), P(f))
        out[f"u32_f32_{lr}"] = f
        a = np.zeros(len(u64))
        R.ref_u01_u64_f64(lr, len(u64), P(u64), P(a))
        out[f"u64_f64_{lr}"] = a
    return out


def dists(R):
    out = {}
    key = np.array([5, 7, 0, 0], np.uint64)
    ctr = np.array([3, 1, 0, 0], np.uint64)
    for eng in (0, 1):
        for batch in (0, 1):
            for n in (7, 1025, 3001):
                a = np.zeros(n)
                R.ref_u01_dist_f64(eng, P(key), P(ctr), n, P(a), batch)
                out[f"u01_e{eng}_b{batch}_n{n}"] = a.copy()
                R.ref_normal_f64(eng, P(key), P(ctr), n, 1.5, 2.0, P(a), batch)
                out[f"normal_e{eng}_b{batch}_n{n}"] = a.copy()
                f = np.zeros(n, np.float32)
                R.ref_normal_f32(eng, P(key), P(ctr), n, 1.5, 2.0, P(f), batch)
                out[f"normalf_e{eng}_b{batch}_n{n}"] = f
        for df in (0.2, 1.0, 1.5, 2.0, 3.0, 10.0, 30.0):
            a = np.zeros(500)
            R.ref_student_t_f64(eng, P(key), P(ctr), 500, df, P(a), 0)
            out[f"student_t_e{eng}_df{df}"] = a
            # the batch form (student_t_distribution, as vsmc_rng_student_t
            # calls it): gamma algorithms T (0.2), W (1.5), E (2), N (3, 10)
            if df not in (0.2, 1.5, 2.0, 3.0, 10.0):
                continue
            for n in (1, 7, 1025, 2049):
                b = np.zeros(n)
                R.ref_student_t_f64(eng, P(key), P(ctr), n, df, P(b), 1)
                out[f"student_t_batch_e{eng}_df{df}_n{n}"] = b
    out.update(key=key, ctr=ctr)
    return out


def sequences(R):
    out = {}
    k2 = np.array([9, 11], np.uint32)
    c4 = np.array([0xFFFFFFF0, 2, 0, 0], np.uint32)
    for kind in range(3):
        for N in (1, 2, 5, 1000):
            a = np.zeros(N)
            nxt = np.zeros(4, np.uint32)
            R.ref_u01_sequence(kind, N, P(k2), P(c4), P(a), P(nxt))
            out[f"seq{kind}_n{N}"] = a
            out[f"seq{kind}_n{N}_next"] = nxt
    out.update(key=k2, ctr=c4)
    return out


def resampling(R, rng):
    out = {}
    k2 = np.array([9, 11], np.uint32)
    c4 = np.array([0xFFFFFFF0, 2, 0, 0], np.uint32)
    sizes = [(1, 5), (5, 0), (2, 3), (100, 100), (1000, 1000), (1000, 700),
             (20000, 20000)]
    for si, (M, N) in enumerate(sizes):
        lw = rng.normal(0, 3, M)
        w = np.exp(lw - lw.max())
        w /= w.sum()
        out[f"w{si}"] = w
        out[f"mn{si}"] = np.array([M, N])
        u = np.sort(rng.random(max(N, 1))[:N])
        out[f"u{si}"] = u
        rep = np.zeros(M, np.int32)
        R.vsmc_resample_trans_u01_rep(M, N, P(w), P(u), P(rep))
        out[f"u01rep{si}"] = rep
        for scheme in range(6):
            rep = np.zeros(M, np.int32)
            nxt = np.zeros(4, np.uint32)
            R.ref_resample(scheme, M, N, P(k2), P(c4), P(w), P(rep), P(nxt))
            out[f"scheme{scheme}_{si}"] = rep
            out[f"scheme{scheme}_{si}_next"] = nxt
            if M == N and M > 1:
                idx = np.zeros(N, np.int32)
                R.vsmc_resample_trans_rep_index(M, N, P(rep), P(idx))
                out[f"scheme{scheme}_{si}_idx"] = idx
        resid = np.zeros(M)
        integ = np.zeros(M, np.int32)
        out[f"residR{si}"] = np.array(
            [R.vsmc_resample_trans_residual(M, max(N, 1), P(w), P(resid),
                                            P(integ))])
        out[f"resid{si}"] = resid
        out[f"integ{si}"] = integ
    out.update(key=k2, ctr=c4, nsizes=np.array([len(sizes)]))
    return out


def weights(R, rng):
    out = {}
    for n in (1, 3, 1025, 5000):
        lw = rng.normal(0, 3, n)
        W = np.zeros(n)
        ess = R.ref_weight_set_log(n, P(lw), P(W))
        l = rng.normal(0, 1, n)
        W2 = np.zeros(n)
        ess2 = R.ref_weight_add_log(n, P(W), P(l), P(W2))
        w = rng.random(n) + 0.01
        W3 = np.zeros(n)
        ess3 = R.ref_weight_set(n, P(w), P(W3))
        out.update({f"lw{n}": lw, f"W{n}": W, f"ess{n}": np.array([ess]),
                    f"l{n}": l, f"W2_{n}": W2, f"ess2_{n}": np.array([ess2]),
                    f"w{n}": w, f"W3_{n}": W3, f"ess3_{n}": np.array([ess3])})
    return out


def pf_runs(R):
    m = (0.1, 1.0, 0.5, 10.0, 2.0, 1.0)
    out = {}
    T = 100
    truth = np.zeros(4 * T)
    obs = np.zeros(2 * T)
    R.ref_pf_simulate(0, T, *m, P(truth), P(obs))
    out["truth"] = truth.reshape(T, 4)
    out["obs"] = obs.reshape(T, 2)
    # the (key = step, counter = particle) streams: trajectories to compare
    for prec in (64, 32):
        for scheme in (1, 2):
            n, TT = 4096, 50
            mean = np.zeros(2 * TT)
            ess = np.zeros(TT)
            res = np.zeros(TT, np.int32)
            logz = np.zeros(TT)
            R.ref_pf_run(prec, n, TT, 3, scheme, 0.5, 0, *m, P(obs), P(mean),
                         P(ess), P(res), P(logz))
            tag = f"p{prec}_s{scheme}"
            out[f"{tag}_mean"] = mean.reshape(TT, 2)
            out[f"{tag}_ess"] = ess
            out[f"{tag}_res"] = res
            out[f"{tag}_logz"] = logz
    # the reference's own per-particle engines: config 1 over 64 runs.
    # Seed::get() steps the global seed by one per engine (rng/seed.hpp:
    # 118-176), so the N particle engines of a run started at seed s take
    # s + 1 .. s + N: runs started one apart would share N - 1 of their
    # particles.  The runs start N + 64 apart, so no engine is shared.
    N = 1 << 14
    seeds = np.arange(64, dtype=np.uint32) * np.uint32(N + 64)
    logz_end = np.zeros(64)
    mean_all = np.zeros((64, T, 2))
    for k, seed in enumerate(seeds):
        mean = np.zeros(2 * T)
        ess = np.zeros(T)
        res = np.zeros(T, np.int32)
        logz = np.zeros(T)
        R.ref_pf_run(64, N, T, int(seed), 1, 0.5, 1, *m, P(obs), P(mean),
                     P(ess), P(res), P(logz))
        logz_end[k] = logz[-1]
        mean_all[k] = mean.reshape(T, 2)
    out["native64_seeds"] = seeds
    out["native64_logz"] = logz_end
    out["native64_mean_avg"] = mean_all.mean(axis=0)
    out["native64_mean_sd"] = mean_all.std(axis=0, ddof=1)
    return out


def genealogy(R, rng):
    """ResampleIndex (resample/index.hpp) traces and index matrices over
    random index histories, and Sampler::print (core/sampler.hpp:646-689)
    of a short FP64 filter run with its histories."""
    out = {}
    for si, (N, iters) in enumerate([(1, 1), (7, 1), (13, 5), (200, 17)]):
        rows = np.zeros((iters, N), np.int32)
        for it in range(iters):
            if rng.random() < 0.3:
                rows[it] = np.arange(N)  # a step without resampling
            else:
                rows[it] = np.sort(rng.integers(0, N, N))
        out[f"rows{si}"] = rows
        for layout in (0, 1):
            m = np.zeros(N * iters, np.int32)
            tr = np.zeros(N * iters, np.int32)
            R.ref_resample_index(N, iters, P(rows), layout, P(m), P(tr))
            out[f"matrix{si}_{layout}"] = m
            out[f"trace{si}"] = tr
    out["nsizes"] = np.array([4])
    m = (0.1, 1.0, 0.5, 10.0, 2.0, 1.0)
    T, N = 20, 1000
    truth = np.zeros(4 * T)
    obs = np.zeros(2 * T)
    R.ref_pf_simulate(2, T, *m, P(truth), P(obs))
    mean = np.zeros(2 * T)
    ess = np.zeros(T)
    res = np.zeros(T, np.int32)
    logz = np.zeros(T)
    buf = ctypes.create_string_buffer(1 << 16)
    n = R.ref_pf_print(N, T, 7, 1, 0.5, *m, P(obs), P(mean), P(ess), P(res),
                       P(logz), buf, len(buf))
    assert n < len(buf)
    out.update(tsv=np.frombuffer(buf.raw[:n], np.uint8), tsv_N=np.array([N]),
               tsv_mean=mean.reshape(T, 2), tsv_ess=ess, tsv_res=res)
    return out


def main(only=None):
    if binding.build_ref() is None:
        sys.exit("reference tree not found: cannot generate the fixtures")
    R = binding.ref()
    rng = np.random.default_rng(20261203)
    for name, fn in (("rng_words", lambda: rng_words(R)),
                     ("u01", lambda: u01(R, rng)),
                     ("dist", lambda: dists(R)),
                     ("sequences", lambda: sequences(R)),
                     ("resample", lambda: resampling(R, rng)),
                     ("weight", lambda: weights(R, rng)),
                     ("pf", lambda: pf_runs(R)),
                     ("genealogy", lambda: genealogy(R, rng))):
        if only and name not in only:
            # keep the draws of the shared generator in their order
            if name in ("u01", "resample", "weight", "genealogy"):
                fn()
            continue
        data = fn()
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **data)
        print(f"{path}: {len(data)} arrays, {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    # optional arguments: the fixture names to write (default all)
    main(set(sys.argv[1:]) or None)
