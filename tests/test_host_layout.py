"""The host plans of the hot path, checked on the CPU: the linearization's scatter plan against an
independent count, and the Schur plan against a dense Schur complement.

The plan (symforce_gb300/csrc/host_layout.cpp, the block analogue of
Linearizer::BuildInitialLinearization, symforce/opt/linearizer.cc:148-356) gives every factor
entry a sink index: a Hessian / rhs value written in place, or a staging slot summed later; a warp
of 32 reprojection factors of one camera sums its camera entries and stores them once.  Here the
device's scatter is replayed in numpy with every factor entry worth 1 (a merged warp's sum worth
32): each in-place value and each staging slot must be written exactly once, and after the staged
sums every Hessian / rhs value must equal the number of factors that touch it, counted directly
from the factors' keys and the block pattern (no use of the plan).  The library's host sources are
compiled with g++ beside a small shim (tests/host_layout_shim.cpp) that hands the plans out."""

from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from symforce_gb300 import _cabi as A
from symforce_gb300 import synth

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "symforce_gb300" / "csrc"
MERGED_KEY_SLOTS = {A.SFG_FACTOR_SNAVELY_REPROJECTION: 2}  # MergedKeySlots in common.h


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    gxx = shutil.which("g++")
    cuda_inc = Path("/usr/local/cuda/include")
    if gxx is None or not (cuda_inc / "cuda_runtime.h").exists():
        pytest.skip("g++ or the CUDA headers are not available")
    out = tmp_path_factory.mktemp("shim") / "libhostshim.so"
    srcs = [ROOT / "tests" / "host_layout_shim.cpp"] + [CSRC / f for f in
                                                        ("host_structure.cpp", "host_layout.cpp", "host_pcg.cpp")]
    subprocess.run([gxx, "-O1", "-std=c++17", "-shared", "-fPIC", "-pthread", f"-I{cuda_inc}", f"-I{ROOT / 'include'}",
                    f"-I{CSRC}", *map(str, srcs), "-o", str(out)], check=True)
    lib = C.CDLL(str(out))
    lib.shim_build.argtypes = [C.POINTER(A.ProblemC)]
    return lib


def _arr(n, dtype):
    return np.zeros(int(n), dtype=dtype)


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _expected_counts(p: A.ProblemArrays, colptr, rows, boff, toff, nvals, N):
    """Contributions of every Hessian value and rhs entry, from the keys and the block pattern."""
    tdim = np.array([A.KEY_DIMS[int(t)][1] for t in p.key_types])
    block = {}
    for j in range(len(colptr) - 1):
        for q in range(colptr[j], colptr[j + 1]):
            block[(int(rows[q]), j)] = int(boff[q])
    cnt = np.zeros(nvals + N, dtype=np.int64)
    for b in p.batches:
        for keys in np.asarray(b.keys):
            cols = [(int(k), r) for k in keys for r in range(tdim[k])]
            for a, (ka, ra) in enumerate(cols):
                for (kb, rb) in cols[:a + 1]:
                    if ka == kb:
                        cnt[block[(ka, ka)] + ra * tdim[ka] + rb] += 1
                    elif ka > kb:
                        cnt[block[(ka, kb)] + ra * tdim[kb] + rb] += 1
                    else:
                        cnt[block[(kb, ka)] + rb * tdim[ka] + ra] += 1
                cnt[nvals + toff[ka] + ra] += 1
    return cnt


def _replay(lib, p: A.ProblemArrays):
    c = p.to_c()
    assert lib.shim_build(C.byref(c)) == 0
    sizes = _arr(7, np.int64)
    lib.shim_sizes(_ptr(sizes))
    nvals, N, nstage, ngroups, nbatches, nblocks, nkeys = (int(x) for x in sizes)
    colptr, rows, boff, toff = _arr(nkeys + 1, np.int64), _arr(nblocks, np.int32), _arr(nblocks, np.int64), \
        _arr(nkeys + 1, np.int64)
    lib.shim_pattern(_ptr(colptr), _ptr(rows), _ptr(boff), _ptr(toff))
    red_dst, red_ptr = _arr(ngroups, np.int32), _arr(ngroups + 1, np.int64)
    lib.shim_groups(_ptr(red_dst), _ptr(red_ptr))
    tdim = np.array([A.KEY_DIMS[int(t)][1] for t in p.key_types])

    value = np.zeros(nvals + N, dtype=np.int64)
    writes = np.zeros(nvals + N, dtype=np.int64)
    stage = np.zeros(nstage, dtype=np.int64)
    stage_writes = np.zeros(nstage, dtype=np.int64)
    merged_warps = 0
    for bi, b in enumerate(p.batches):
        info = _arr(3, np.int32)
        lib.shim_batch(bi, _ptr(info))
        nent, mt, count = (int(x) for x in info)
        dest, order = _arr(nent * count, np.int32), _arr(count, np.int32)
        lib.shim_batch_arrays(bi, _ptr(dest), _ptr(order))
        dest = dest.reshape(nent, count)
        assert sorted(order.tolist()) == list(range(count))
        keys = np.asarray(b.keys)[order]  # device order
        ms = MERGED_KEY_SLOTS.get(b.kind, 0)
        assert mt == sum(tdim[keys[0, s]] for s in range(ms)) if count else True
        td = sum(tdim[k] for k in keys[0]) if count else 0
        nh = td * (td + 1) // 2
        merged_entry = np.array([(e < mt * (mt + 1) // 2) if e < nh else (e - nh < mt) for e in range(nent)])
        for f in range(count):
            w0 = f - f % 32
            merged = (ms > 0 and w0 + 32 <= count
                      and all((keys[w0:w0 + 32, s] == keys[w0, s]).all() for s in range(ms)))
            if merged and f == w0:
                merged_warps += 1
            for e in range(nent):
                v = 1
                if merged and merged_entry[e]:
                    if f != w0:
                        continue
                    v = 32
                d = int(dest[e, f])
                if d < nvals + N:
                    value[d] += v
                    writes[d] += 1
                else:
                    stage[d - nvals - N] += v
                    stage_writes[d - nvals - N] += 1
    assert (writes <= 1).all(), "a value written in place by two contributions"
    assert (stage_writes == 1).all(), "a staging slot not written exactly once"
    for g in range(ngroups):
        s = int(red_dst[g])
        assert writes[s] == 0, "a staged destination also written in place"
        value[s] = stage[red_ptr[g]:red_ptr[g + 1]].sum()
    expected = _expected_counts(p, colptr, rows, boff, toff, nvals, N)
    np.testing.assert_array_equal(value, expected)
    return merged_warps


def test_reprojection_plan_with_merged_warps(shim):
    # ~100 observations per camera: whole warps of one camera (merged) and mixed warps at the ends
    p = synth.bundle_adjustment(num_cameras=6, num_points=150, num_observations=620, seed=2)
    assert _replay(shim, p) > 0


def test_plans_without_merging(shim):
    assert _replay(shim, synth.robot_2d(num_poses=60, num_landmarks=8, seed=3)) == 0
    assert _replay(shim, synth.pose3_chain(num_poses=40, num_landmarks=12, seed=4)) == 0


def _schur_arrays(lib):
    sizes = _arr(9, np.int64)
    lib.shim_schur_sizes(_ptr(sizes))
    nbk, npts, nB, c_toff, nE, nsb, nterms, nr, nS = (int(x) for x in sizes)
    n64 = {0: npts, 1: npts + 1, 2: nE, 3: nE, 4: nsb + 1, 5: nterms, 6: nterms, 7: nsb, 8: nsb,
           9: nB + 1, 10: nr, 11: nbk + 1, 12: nsb}
    n32 = {0: nE, 1: nsb, 2: nsb, 3: nr, 4: nr, 5: nr, 6: nsb}
    a64, a32 = {}, {}
    for k, n in n64.items():
        a64[k] = _arr(n, np.int64)
        lib.shim_schur_i64(k, _ptr(a64[k]))
    for k, n in n32.items():
        a32[k] = _arr(n, np.int32)
        lib.shim_schur_i32(k, _ptr(a32[k]))
    return (nbk, npts, nB, c_toff, nS), a64, a32


@pytest.mark.parametrize("g_at_e", [False, True])
def test_schur_plan_matches_dense_schur_complement(shim, g_at_e):
    """The Schur plan (point C blocks, per-S-block term lists, reduced-rhs lists) replayed in numpy
    on random block values gives S = B - E^T C^-1 E (as sum G_pk^T G_pl, G = L^-1 E) and
    v = g_B - E^T C^-1 g_C of the dense matrix (symforce/opt/sparse_schur_solver.tcc:15-170)."""
    p = synth.bundle_adjustment(num_cameras=5, num_points=60, num_observations=240, seed=7)
    c = p.to_c()
    assert shim.shim_build(C.byref(c)) == 0 and shim.shim_build_schur() == 0
    sizes = _arr(7, np.int64)
    shim.shim_sizes(_ptr(sizes))
    nvals, N, _, _, _, nblocks, nkeys = (int(x) for x in sizes)
    if g_at_e:  # G at E's offsets; the G kernel's order visits every E block once, offsets ascending
        ssz = _arr(9, np.int64)
        shim.shim_schur_sizes(_ptr(ssz))
        order = _arr(int(ssz[4]), np.int64)
        assert shim.shim_build_schur_g_at_e(_ptr(order)) == 0
        assert sorted(order.tolist()) == list(range(len(order)))
    colptr, rows, boff, toff = _arr(nkeys + 1, np.int64), _arr(nblocks, np.int32), _arr(nblocks, np.int64), \
        _arr(nkeys + 1, np.int64)
    shim.shim_pattern(_ptr(colptr), _ptr(rows), _ptr(boff), _ptr(toff))
    tdim = np.diff(toff)
    rng = np.random.default_rng(1)
    vals = rng.normal(size=nvals)
    H = np.zeros((N, N))
    for j in range(nkeys):
        for q in range(colptr[j], colptr[j + 1]):
            i = int(rows[q])
            blk = vals[boff[q]:boff[q] + tdim[i] * tdim[j]].reshape(tdim[i], tdim[j])
            if i == j:  # symmetric diagonal blocks, stored full
                blk = np.tril(blk) + np.tril(blk, -1).T + 12.0 * np.eye(tdim[i])
                vals[boff[q]:boff[q] + tdim[i] * tdim[j]] = blk.ravel()
            H[toff[i]:toff[i] + tdim[i], toff[j]:toff[j] + tdim[j]] = blk
            H[toff[j]:toff[j] + tdim[j], toff[i]:toff[i] + tdim[i]] = blk.T
    g = rng.normal(size=N)

    (nbk, npts, nB, c_toff, nS), a64, a32 = _schur_arrays(shim)
    assert nB == toff[nbk] and c_toff == nB
    # replay: L^-1 (C = L L^T) and t per point, G = L^-1 E per E block (at E's offset), S blocks
    # from their terms (G_pk^T G_pl), v from its lists
    Cs = [vals[a64[0][q]:a64[0][q] + 9].reshape(3, 3) for q in range(npts)]
    linv = [np.linalg.inv(np.linalg.cholesky(Cq)) for Cq in Cs]
    t = np.array([np.linalg.solve(Cs[q], g[c_toff + 3 * q:c_toff + 3 * q + 3]) for q in range(npts)])
    goff = a64[2] if g_at_e else a64[3]  # where each block's G lives
    if g_at_e:
        assert np.all(np.diff(a64[2][order]) > 0)
    Wv = np.zeros(int(max(goff[e] + 3 * a32[0][e] for e in range(len(goff)))))
    for q in range(npts):
        for e in range(a64[1][q], a64[1][q + 1]):
            dk = int(a32[0][e])
            E = vals[a64[2][e]:a64[2][e] + 3 * dk].reshape(3, dk)
            Wv[goff[e]:goff[e] + 3 * dk] = (linv[q] @ E).ravel()
    Sv = np.zeros(nS)
    for q in range(len(a64[7])):
        dk, dl = int(a32[1][q]), int(a32[2][q])
        acc = np.zeros((dk, dl))
        for u in range(a64[4][q], a64[4][q + 1]):
            Gk = Wv[a64[5][u]:a64[5][u] + 3 * dk].reshape(3, dk)
            Gl = Wv[a64[6][u]:a64[6][u] + 3 * dl].reshape(3, dl)
            acc += Gk.T @ Gl
        B = vals[a64[7][q]:a64[7][q] + dk * dl].reshape(dk, dl) if a64[7][q] >= 0 else 0.0
        Sv[a64[8][q]:a64[8][q] + dk * dl] = (B - acc).ravel()
    v = g[:nB].copy()
    for i in range(nB):
        for u in range(a64[9][i], a64[9][i + 1]):
            dk, col, pt = int(a32[4][u]), int(a32[3][u]), int(a32[5][u])
            E = vals[a64[10][u] + col + dk * np.arange(3)]
            v[i] -= E @ t[pt]
    # dense reference
    Cinv = np.linalg.inv(H[nB:, nB:])
    Sd = H[:nB, :nB] - H[:nB, nB:] @ Cinv @ H[nB:, :nB]
    vd = g[:nB] - H[:nB, nB:] @ Cinv @ g[nB:]
    np.testing.assert_allclose(v, vd, rtol=1e-10, atol=1e-10)
    scol, srow, sboff = a64[11], a32[6], a64[12]
    checked = 0
    for j in range(nbk):
        for q in range(scol[j], scol[j + 1]):
            i = int(srow[q])
            blk = Sv[sboff[q]:sboff[q] + tdim[i] * tdim[j]].reshape(tdim[i], tdim[j])
            ref = Sd[toff[i]:toff[i] + tdim[i], toff[j]:toff[j] + tdim[j]]
            np.testing.assert_allclose(blk, ref, rtol=1e-10, atol=1e-10)
            checked += 1
    assert checked == len(a64[7])
    # every nonzero of the dense lower S lies in a stored block
    mask = np.zeros((nB, nB), dtype=bool)
    for j in range(nbk):
        for q in range(scol[j], scol[j + 1]):
            i = int(srow[q])
            mask[toff[i]:toff[i] + tdim[i], toff[j]:toff[j] + tdim[j]] = True
    assert np.abs(np.tril(Sd)[~mask]).max(initial=0.0) < 1e-12


# tile task types of the persistent factorization (device.cuh TaskType)
ASSEMBLE, DIAG, TRSM, UPDATE, LOOKAHEAD, CHAIN, INVERSE, UPDATE_TC = 0, 1, 2, 3, 4, 5, 6, 7
FINAL = 1 << 30


def _factor_plan(lib, which, tile):
    assert lib.shim_build_factor_plan(which, tile) == 0
    sizes = _arr(3, np.int64)
    lib.shim_factor_sizes(_ptr(sizes))
    ns, ntasks, nc = (int(x) for x in sizes)
    tasks = _arr(4 * ntasks, np.int32)
    npiv, ntiles, parent, w, m = (_arr(ns, np.int32) for _ in range(5))
    cptr, clist = _arr(ns + 1, np.int32), _arr(nc, np.int32)
    lib.shim_factor_arrays(*(_ptr(a) for a in (tasks, npiv, ntiles, parent, w, m, cptr, clist)))
    return tasks.reshape(ntasks, 4), npiv, ntiles, parent, w, m, cptr, clist


def _replay_tasks(tasks, npiv, ntiles, parent, w, m, cptr, clist, tile):
    """Run the task list in its own order on the tile-state machine of the factorization kernel
    (kernels_solve.cu: TaskAssemble, TaskDiag, TaskTrsm, TaskLookahead, TaskUpdate, TaskChain,
    TaskInverse): every wait must already hold when its task comes up.  The kernel's CTAs claim
    tasks in list order, so a task only ever waits on tasks claimed before it, which then always
    finish.  A chain task stays in its CTA for the front's whole factorization: its steps are run
    here as soon as their waits hold (the chain's CTA advances by itself), and a later task that
    waits on a step that cannot have run yet fails the replay; every chain must end up complete.
    So no task waits on a step that waits on an unclaimed task: no deadlock.  (A CTA claims its
    next task when it starts one, except under a chain task, whose CTA would otherwise hold a task
    the chain waits on.)"""
    ns = len(npiv)
    state = [np.zeros((int(ntiles[s]), int(ntiles[s])), dtype=np.int64) for s in range(ns)]
    chains = {}  # front -> next chain step (-1: the diagonal tile (0, 0))

    def need(s, i, j, v, what):
        assert state[s][i, j] >= v, f"front {s}: {what} waits on tile ({i}, {j}) >= {v}, has {state[s][i, j]}"

    def advance_chains():
        for s in list(chains):
            st, nps = state[s], int(npiv[s])
            while True:
                k = chains[s]
                if k < 0:
                    if st[0, 0] < 1:
                        break
                    st[0, 0] = FINAL
                else:
                    # step k: the panel solve of (k+1, k), the update of (k+1, k+1) by it and its
                    # LDL^T
                    i = k + 1
                    assert st[k, k] == FINAL
                    if st[i, k] < 1 + k or st[i, i] < 1 + k:
                        break
                    st[i, k] = FINAL
                    st[i, i] = FINAL
                chains[s] = k + 1
                if chains[s] + 1 >= nps:
                    del chains[s]
                    break

    for ty, s, z, kw in tasks:
        advance_chains()
        i, j = int(z) >> 16, int(z) & 0xFFFF
        k, cnt = int(kw) & 0xFFFFF, int(kw) >> 20
        st = state[s]
        if ty == CHAIN:
            assert int(npiv[s]) > 1 and s not in chains
            chains[s] = -1
            advance_chains()
        elif ty == INVERSE:
            assert i == j == k
            need(s, k, k, FINAL, "inverse")
        elif ty == ASSEMBLE:
            for c in clist[cptr[s]:cptr[s + 1]]:
                npc, ntc = int(npiv[c]), int(ntiles[c])
                for a in range(npc, ntc):
                    for b in range(npc, a + 1):
                        need(c, a, b, 1 + npc, "assemble")
            st[j:, j] = 1
        elif ty == DIAG:
            need(s, k, k, 1 + k, "diag")
            st[k, k] = FINAL
        elif ty == TRSM or ty == LOOKAHEAD:
            need(s, k, k, FINAL, "panel")
            need(s, i, k, 1 + k, "panel")
            st[i, k] = FINAL
            if ty == LOOKAHEAD:
                # the FP64 look-ahead waits for this one at its start, the FP32 one after its panel
                # solve; (i, i) does not depend on (i, k), so the replay is the same for both
                assert i == k + 1
                need(s, i, i, 1 + k, "lookahead diag")
                st[i, i] = FINAL
        elif ty == UPDATE:
            need(s, i, k, FINAL, "update")
            need(s, j, k, FINAL, "update")
            need(s, i, j, 1 + k, "update")
            st[i, j] = 2 + k
        elif ty == UPDATE_TC:
            assert 2 <= cnt <= 4
            need(s, j, k, FINAL, "tensor-core update")
            for r in range(i, i + cnt):
                need(s, r, k, FINAL, "tensor-core update")
                need(s, r, j, 1 + k, "tensor-core update")
                st[r, j] = 2 + k
        else:
            raise AssertionError(f"unknown task type {ty}")
    advance_chains()
    assert not chains, f"chains left unfinished: {chains}"
    # every front fully factored: pivot and panel tiles final, the update block through all panels
    for s in range(ns):
        nps, nts = int(npiv[s]), int(ntiles[s])
        assert nps == -(-int(w[s]) // tile) and nts == nps + -(-(int(m[s]) - int(w[s])) // tile)
        for a in range(nts):
            for b in range(min(a + 1, nps)):
                assert state[s][a, b] == FINAL, (s, a, b)
            for b in range(nps, a + 1):
                assert state[s][a, b] == 1 + nps, (s, a, b)
        # postorder: the forward solve runs fronts in order, the backward solve in reverse
        assert parent[s] == -1 or parent[s] > s


@pytest.mark.parametrize("tile", [16, 32])
def test_factor_task_plan_is_deadlock_free(shim, tile):
    """The tile task lists of the reduced camera system (bundle adjustment) and of a full Hessian
    (2D localization, no Schur) pass the replay at both tile sizes (FP64 16, FP32 32)."""
    p = synth.bundle_adjustment(num_cameras=80, num_points=2000, num_observations=8000, seed=5)
    c = p.to_c()
    assert shim.shim_build(C.byref(c)) == 0 and shim.shim_build_schur() == 0
    plan = _factor_plan(shim, 1, tile)
    assert len(plan[1]) > 1  # several fronts: the assembly waits on children are exercised
    _replay_tasks(*plan, tile)
    r = synth.robot_2d(num_poses=300, num_landmarks=12, seed=6)
    c2 = r.to_c()
    assert shim.shim_build(C.byref(c2)) == 0
    _replay_tasks(*_factor_plan(shim, 0, tile), tile)


def _maps(lib):
    sizes = _arr(14, np.int64)
    lib.shim_maps_sizes(_ptr(sizes))
    n64 = {0: 0, 1: 1, 2: 2, 3: 3, 4: 4, 5: 5, 7: 7, 9: 9}
    n32 = {21: 1, 22: 1, 24: 4, 26: 6, 28: 8, 30: 10, 31: 11}
    out = {}
    for k, sz in n64.items():
        out[k] = _arr(sizes[sz], np.int64)
        lib.shim_maps_i64(k, _ptr(out[k]))
    for k, sz in n32.items():
        out[k] = _arr(sizes[sz], np.int32)
        lib.shim_maps_i32(k, _ptr(out[k]))
    return out, int(sizes[12]), int(sizes[13])


def _dense_from_pattern(colptr, rows, boff, off, rng):
    """Random diagonally dominant symmetric values on a block pattern (lower blocks row-major,
    diagonal blocks stored full) and the dense matrix they stand for."""
    dims = np.diff(off)
    vals = np.zeros(max(int(boff[q] + dims[rows[q]] * dims[j]) for j in range(len(colptr) - 1)
                        for q in range(colptr[j], colptr[j + 1])))
    n = int(off[-1])
    A = np.zeros((n, n))
    for j in range(len(colptr) - 1):
        for q in range(colptr[j], colptr[j + 1]):
            i = int(rows[q])
            blk = rng.normal(size=(dims[i], dims[j]))
            if i == j:
                blk = np.tril(blk) + np.tril(blk, -1).T
            vals[boff[q]:boff[q] + blk.size] = blk.ravel()
            A[off[i]:off[i] + dims[i], off[j]:off[j] + dims[j]] = blk
            A[off[j]:off[j] + dims[j], off[i]:off[i] + dims[i]] = blk.T
    shift = np.abs(A).sum(axis=1) + 1.0  # dominance through the damping
    return vals, A, shift


def _replay_numeric(plan, mp, pool, n, vals, damping, b):
    """The multifrontal LDL^T and solve of the device, replayed in numpy from the host maps: each
    front assembled from the matrix values (+ damping on the diagonal) and its children's update
    blocks, its pivot columns factored, then the forward and backward solves by front."""
    tasks, npiv, ntiles, parent, w, m, cptr, clist = plan
    col_base, a_ptr, a_src, a_dst, a_damp = mp[31], mp[0], mp[1], mp[21], mp[22]
    e_rptr, e_round, e_src, e_dst = mp[2], mp[3], mp[4], mp[24]
    idx_off, idx, rel_off, rel, foff, scalar_old = mp[5], mp[26], mp[7], mp[28], mp[9], mp[30]
    F = np.zeros(pool)
    ns = len(w)
    fronts = []
    for s in range(ns):
        ms, ws, base = int(m[s]), int(w[s]), int(foff[s])
        for slot in range(col_base[s], col_base[s + 1]):
            for e in range(a_ptr[slot], a_ptr[slot + 1]):
                v = vals[a_src[e]] + (damping[a_damp[e]] if a_damp[e] >= 0 else 0.0)
                F[base + a_dst[e]] = v
            for rd in range(e_rptr[slot], e_rptr[slot + 1]):
                for e in range(e_round[rd], e_round[rd + 1]):
                    F[base + e_dst[e]] += F[e_src[e]]
        Fm = F[base:base + ms * ms].reshape(ms, ms).T.copy()  # column-major front
        Fm = np.tril(Fm) + np.tril(Fm, -1).T
        for j in range(ws):
            col = Fm[j + 1:, j].copy()
            lj = col / Fm[j, j]
            Fm[j + 1:, j + 1:] -= np.outer(lj, col)
            Fm[j + 1:, j] = lj
        F[base:base + ms * ms] = Fm.T.ravel()
        fronts.append(Fm)
    ycon, ysave, xperm, x = np.zeros(rel_off[-1]), np.zeros(idx_off[-1]), np.zeros(n), np.zeros(n)
    for s in range(ns):
        ms, ws = int(m[s]), int(w[s])
        ids = idx[idx_off[s]:idx_off[s] + ms]
        xs = np.zeros(ms)
        xs[:ws] = b[scalar_old[ids[:ws]]]
        for c in clist[cptr[s]:cptr[s + 1]]:
            hc = int(m[c] - w[c])
            xs[rel[rel_off[c]:rel_off[c] + hc]] += ycon[rel_off[c]:rel_off[c] + hc]
        L = np.tril(fronts[s][:ws, :ws], -1) + np.eye(ws)
        y = np.linalg.solve(L, xs[:ws])
        xs[ws:] -= fronts[s][ws:, :ws] @ y
        ysave[idx_off[s]:idx_off[s] + ws] = y
        ycon[rel_off[s]:rel_off[s] + ms - ws] = xs[ws:]
    for s in reversed(range(ns)):
        ms, ws = int(m[s]), int(w[s])
        ids = idx[idx_off[s]:idx_off[s] + ms]
        L = np.tril(fronts[s][:ws, :ws], -1) + np.eye(ws)
        z = ysave[idx_off[s]:idx_off[s] + ws] / np.diag(fronts[s])[:ws] - fronts[s][ws:, :ws].T @ xperm[ids[ws:]]
        xp = np.linalg.solve(L.T, z)
        xperm[ids[:ws]] = xp
        x[scalar_old[ids[:ws]]] = xp
    return x


def test_factor_maps_solve_the_system(shim):
    """The assembly lists, extend-add rounds and solve maps of the factorization plan, replayed in
    numpy on random values, solve (A + diag(damping)) x = b as a dense solve does (the reduced BA
    system with several fronts, and a 2D localization Hessian)."""
    rng = np.random.default_rng(3)

    def reduced_ba():
        p = synth.bundle_adjustment(num_cameras=80, num_points=2000, num_observations=8000, seed=5)
        c = p.to_c()
        assert shim.shim_build(C.byref(c)) == 0 and shim.shim_build_schur() == 0
        (nbk, _, _, _, _), a64, a32 = _schur_arrays(shim)
        sizes = _arr(7, np.int64)
        shim.shim_sizes(_ptr(sizes))
        nkeys, nblocks = int(sizes[6]), int(sizes[5])
        hcol, hrows, hboff, toff = _arr(nkeys + 1, np.int64), _arr(nblocks, np.int32), _arr(nblocks, np.int64), \
            _arr(nkeys + 1, np.int64)
        shim.shim_pattern(_ptr(hcol), _ptr(hrows), _ptr(hboff), _ptr(toff))
        return 1, a64[11], a32[6], a64[12], toff[:nbk + 1]

    def localization_hessian():
        c = synth.robot_2d(num_poses=200, num_landmarks=10, seed=8).to_c()
        assert shim.shim_build(C.byref(c)) == 0
        sizes = _arr(7, np.int64)
        shim.shim_sizes(_ptr(sizes))
        nkeys, nblocks = int(sizes[6]), int(sizes[5])
        colptr, rows, boff, off = _arr(nkeys + 1, np.int64), _arr(nblocks, np.int32), _arr(nblocks, np.int64), \
            _arr(nkeys + 1, np.int64)
        shim.shim_pattern(_ptr(colptr), _ptr(rows), _ptr(boff), _ptr(off))
        return 0, colptr, rows, boff, off

    for case in (reduced_ba, localization_hessian):
        which, colptr, rows, boff, off = case()
        for tile in (16, 32):
            plan = _factor_plan(shim, which, tile)
            mp, pool, n = _maps(shim)
            assert n == int(off[-1])
            vals, A, shift = _dense_from_pattern(colptr, rows, boff, off, rng)
            b = rng.normal(size=n)
            x = _replay_numeric(plan, mp, pool, n, vals, shift, b)
            ref = np.linalg.solve(A + np.diag(shift), b)
            np.testing.assert_allclose(x, ref, rtol=1e-9, atol=1e-12)


def test_camera_block_rows_give_the_reduced_system_product(shim):
    """The PCG camera-block layout (symforce_gb300/csrc/host_pcg.cpp): 9 x 9 group blocks gathered
    from S and each group row's entries (stored block, neighbour, transposed) give S x as the dense
    product does, and never read the upper triangle of a diagonal key block (not kept current on
    the device; NaN here)."""
    p = synth.bundle_adjustment(num_cameras=40, num_points=900, num_observations=3600, seed=9)
    c = p.to_c()
    assert shim.shim_build(C.byref(c)) == 0 and shim.shim_build_schur() == 0
    assert shim.shim_build_precond() == 0
    (nbk, _, nB, _, nS), a64, a32 = _schur_arrays(shim)
    sizes = _arr(7, np.int64)
    shim.shim_sizes(_ptr(sizes))
    nkeys, nblocks = int(sizes[6]), int(sizes[5])
    hcol, hrows, hboff, toff = _arr(nkeys + 1, np.int64), _arr(nblocks, np.int32), _arr(nblocks, np.int64), \
        _arr(nkeys + 1, np.int64)
    shim.shim_pattern(_ptr(hcol), _ptr(hrows), _ptr(hboff), _ptr(toff))
    dims = np.diff(toff[:nbk + 1])
    scol, srow, sboff = a64[11], a32[6], a64[12]
    rng = np.random.default_rng(4)
    Sv = np.zeros(nS)
    Sd = np.zeros((nB, nB))
    for j in range(nbk):
        for q in range(scol[j], scol[j + 1]):
            i = int(srow[q])
            blk = rng.normal(size=(dims[i], dims[j]))
            if i == j:
                blk = np.tril(blk) + np.tril(blk, -1).T
                stored = blk.copy()
                stored[np.triu_indices(dims[i], 1)] = np.nan
            else:
                stored = blk
            Sv[sboff[q]:sboff[q] + blk.size] = stored.ravel()
            Sd[toff[i]:toff[i] + dims[i], toff[j]:toff[j] + dims[j]] = blk
            Sd[toff[j]:toff[j] + dims[j], toff[i]:toff[i] + dims[i]] = blk.T
    ps = _arr(3, np.int64)
    shim.shim_precond_sizes(_ptr(ps))
    ng, nbl, nent = (int(x) for x in ps)
    gidx, blk_off = _arr(ng * 9, np.int32), _arr(nbl * 81, np.int64)
    gptr, gent = _arr(ng + 1, np.int32), _arr(2 * nent, np.int32)
    shim.shim_precond_arrays(_ptr(gidx), _ptr(blk_off), _ptr(gptr), _ptr(gent))
    gidx = gidx.reshape(ng, 9)
    assert sorted(gidx[gidx >= 0].tolist()) == list(range(nB))  # every scalar in one block
    Sb = np.where(blk_off >= 0, Sv[np.maximum(blk_off, 0)], 0.0).reshape(nbl, 9, 9)
    x = rng.normal(size=nB)
    xg = np.where(gidx >= 0, x[np.maximum(gidx, 0)], 0.0)
    y = np.zeros((ng, 9))
    for g in range(ng):
        for e in range(gptr[g], gptr[g + 1]):
            blk, nb = int(gent[2 * e]), int(gent[2 * e + 1])
            B = Sb[blk].T if nb & 1 else Sb[blk]
            y[g] += B @ xg[nb >> 1]
    ref = Sd @ x
    ok = gidx >= 0
    np.testing.assert_allclose(y[ok], ref[gidx[ok]], rtol=1e-12, atol=1e-12)
    # band preconditioner pattern: J_l = the groups l - band .. l - 1 that S couples to l, then l;
    # the stored block of every lower pair of J_l
    lower = {}
    for g in range(ng):
        for e in range(gptr[g], gptr[g + 1]):
            blk, nb = int(gent[2 * e]), int(gent[2 * e + 1])
            if not nb & 1:
                lower[(g, nb >> 1)] = blk
    for band in (1, 3):
        k1 = band + 1
        nj, jgrp, jblk = _arr(ng, np.int32), _arr(ng * k1, np.int32), _arr(ng * k1 * k1, np.int32)
        shim.shim_band_pattern(band, _ptr(nj), _ptr(jgrp), _ptr(jblk))
        jgrp, jblk = jgrp.reshape(ng, k1), jblk.reshape(ng, k1, k1)
        for g in range(ng):
            J = [h for h in range(max(0, g - band), g) if (g, h) in lower] + [g]
            assert nj[g] == len(J) and jgrp[g, :len(J)].tolist() == J, (band, g, J)
            for s1 in range(len(J)):
                for s2 in range(s1 + 1):
                    assert jblk[g, s1, s2] == lower.get((J[s1], J[s2]), -1), (band, g, s1, s2)
        assert int(nj.max()) > 1  # some rows do couple to earlier groups


def _random_pose3_graph(rng, nposes, nbetween, nrange):
    """A Pose3 factor graph of random structure (between factors on random pairs, a prior on every
    pose, range factors on random poses): several components, uneven degrees."""
    kt = [A.SFG_KEY_POSE3] * nposes
    pairs = []
    while len(pairs) < nbetween:
        i, j = rng.integers(0, nposes, size=2)
        if i != j:
            pairs.append((int(i), int(j)))
    batches = [A.Batch(A.SFG_FACTOR_BETWEEN_POSE3, np.array(pairs, dtype=np.int32),
                       np.zeros((nbetween, A.FACTOR_DIMS[A.SFG_FACTOR_BETWEEN_POSE3][1]))),
               A.Batch(A.SFG_FACTOR_PRIOR_POSE3, np.arange(nposes, dtype=np.int32)[:, None],
                       np.zeros((nposes, A.FACTOR_DIMS[A.SFG_FACTOR_PRIOR_POSE3][1]))),
               A.Batch(A.SFG_FACTOR_RANGE_POSE3, rng.integers(0, nposes, size=(nrange, 1)).astype(np.int32),
                       np.zeros((nrange, A.FACTOR_DIMS[A.SFG_FACTOR_RANGE_POSE3][1])))]
    values = np.tile(np.array([0, 0, 0, 1, 0, 0, 0], dtype=np.float64), nposes)
    return A.ProblemArrays(key_types=kt, batches=batches, values=values)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_plans_of_random_factor_graphs(shim, seed):
    """Random Pose3 graphs: the scatter plan replays to the factor counts, the task list replays
    without a blocked wait and the factorization maps solve the system, at both tile sizes."""
    rng = np.random.default_rng(100 + seed)
    p = _random_pose3_graph(rng, nposes=int(rng.integers(20, 90)), nbetween=int(rng.integers(30, 200)),
                            nrange=int(rng.integers(0, 60)))
    _replay(shim, p)
    c = p.to_c()
    assert shim.shim_build(C.byref(c)) == 0
    sizes = _arr(7, np.int64)
    shim.shim_sizes(_ptr(sizes))
    nkeys, nblocks = int(sizes[6]), int(sizes[5])
    colptr, rows, boff, off = _arr(nkeys + 1, np.int64), _arr(nblocks, np.int32), _arr(nblocks, np.int64), \
        _arr(nkeys + 1, np.int64)
    shim.shim_pattern(_ptr(colptr), _ptr(rows), _ptr(boff), _ptr(off))
    for tile in (16, 32):
        plan = _factor_plan(shim, 0, tile)
        _replay_tasks(*plan, tile)
        mp, pool, n = _maps(shim)
        vals, Ad, shift = _dense_from_pattern(colptr, rows, boff, off, rng)
        b = rng.normal(size=n)
        x = _replay_numeric(plan, mp, pool, n, vals, shift, b)
        np.testing.assert_allclose(x, np.linalg.solve(Ad + np.diag(shift), b), rtol=1e-9, atol=1e-12)


def _replay_split_solve(fronts, kp, ku, task_front, task_sub, nf, block_tiles, tile, rng):
    """The split front solves of SolveKernel (kernels_solve.cu: OwnsRow, ForwardMulti, BackwardMulti)
    run in task order on random unit-lower fronts.  A value another CTA owns is read from the
    exchange buffer, which holds NaN (the unset pattern) until its owner stores it, so a task that
    needs a value of a later task fails the replay: every wait is on a lower task number.  Each
    front's forward and backward results must equal dense triangular solves."""
    P = block_tiles
    state = {}
    for s, (w, m) in enumerate(fronts):
        np_, nu = -(-w // tile), -(-(m - w) // tile)
        L = np.tril(rng.normal(size=(m, m)) * 0.2, -1) + np.eye(m)
        state[s] = dict(w=w, m=m, np=np_, nt=np_ + nu, L=L, b=rng.normal(size=m), z=rng.normal(size=w),
                        y=np.full(w, np.nan), upd=np.full(m - w, np.nan), xe=np.full(w, np.nan),
                        fwd_done=0, bwd_done=0)

    def owns(st, q, cta, k_p, k_u):
        if k_p == 0:
            return True
        if cta < k_p:
            return q < st["w"] and q // (tile * P) == cta
        return q >= st["w"] and ((q - st["w"]) // tile) % k_u == cta - k_p

    def tstart(st, t):
        return t * tile if t < st["np"] else st["w"] + (t - st["np"]) * tile

    def tsize(st, t):
        return min(tile, st["w"] - t * tile) if t < st["np"] else min(tile, st["m"] - tstart(st, t))

    for t in range(len(task_front)):
        s, c = int(task_front[t]), int(task_sub[t])
        st, k_p, k_u = state[s], int(kp[s]), int(ku[s])
        w, m, np_, nt, L = st["w"], st["m"], st["np"], st["nt"], st["L"]
        if t < nf:
            assert 0 <= c < (k_p + k_u if k_p else 1)
            xs = np.array([st["b"][q] if owns(st, q, c, k_p, k_u) else np.nan for q in range(m)])
            if k_p == 0 or c < k_p:
                tiles = range(np_) if k_p == 0 else range(c * P, min(c * P + P, np_))
                for i in tiles:
                    ri, bi = i * tile, tsize(st, i)
                    for j in range(i):
                        cj, bj = j * tile, tsize(st, j)
                        # earlier blocks' values come from the exchange buffer
                        yj = st["y"][cj:cj + bj] if (k_p == 0 or j < c * P) else xs[cj:cj + bj]
                        assert not np.isnan(yj).any(), f"task {t} waits on an unsolved tile {j}"
                        xs[ri:ri + bi] -= L[ri:ri + bi, cj:cj + bj] @ yj
                    xs[ri:ri + bi] = np.linalg.solve(L[ri:ri + bi, ri:ri + bi], xs[ri:ri + bi])
                    st["y"][ri:ri + bi] = xs[ri:ri + bi]
                if k_p == 0:  # the one-CTA solve also forms the update rows
                    for i in range(np_, nt):
                        ri, bi = tstart(st, i), tsize(st, i)
                        xs[ri:ri + bi] -= L[ri:ri + bi, :w] @ st["y"]
            else:
                for i in range(np_ + (c - k_p), nt, k_u):
                    ri, bi = tstart(st, i), tsize(st, i)
                    assert ri >= w and ri + bi <= m
                    for j in range(np_):
                        cj, bj = j * tile, tsize(st, j)
                        yj = st["y"][cj:cj + bj]
                        assert not np.isnan(yj).any(), f"task {t} waits on an unsolved tile {j}"
                        xs[ri:ri + bi] -= L[ri:ri + bi, cj:cj + bj] @ yj
            for q in range(w, m):
                if owns(st, q, c, k_p, k_u):
                    assert np.isnan(st["upd"][q - w])
                    st["upd"][q - w] = xs[q]
            st["fwd_done"] += 1
        else:
            k_b = k_p if k_p else 1
            assert 0 <= c < k_b
            assert st["fwd_done"] == (k_p + k_u if k_p else 1), f"front {s} backward before its forward"
            blk = k_p - 1 - c
            tiles = range(np_ - 1, -1, -1) if k_p == 0 else range(min(blk * P + P, np_) - 1, blk * P - 1, -1)
            top = np_ - 1 if k_p == 0 else min(blk * P + P, np_) - 1
            xs = st["z"].copy()
            for j in tiles:
                cj, bj = j * tile, tsize(st, j)
                for i in range(np_ - 1, j, -1):
                    ri, bi = i * tile, tsize(st, i)
                    xi = st["xe"][ri:ri + bi] if i > top else xs[ri:ri + bi]
                    assert not np.isnan(xi).any(), f"task {t} waits on an unsolved tile {i}"
                    xs[cj:cj + bj] -= L[ri:ri + bi, cj:cj + bj].T @ xi
                xs[cj:cj + bj] = np.linalg.solve(L[cj:cj + bj, cj:cj + bj].T, xs[cj:cj + bj])
                assert np.isnan(st["xe"][cj:cj + bj]).all()
                st["xe"][cj:cj + bj] = xs[cj:cj + bj]
            st["bwd_done"] += 1
    for s, st in state.items():
        w, L = st["w"], st["L"]
        ref = np.linalg.solve(L[:w, :w], st["b"][:w])
        np.testing.assert_allclose(st["y"], ref, rtol=1e-9, atol=1e-11)
        np.testing.assert_allclose(st["upd"], st["b"][w:] - L[w:, :w] @ ref, rtol=1e-9, atol=1e-11)
        np.testing.assert_allclose(st["xe"], np.linalg.solve(L[:w, :w].T, st["z"]), rtol=1e-9, atol=1e-11)


@pytest.mark.parametrize("warps,block_tiles", [(8, 4), (2, 1), (2, 2), (3, 3)])
def test_split_front_solves(shim, warps, block_tiles):
    """Fronts with more tiles than a solve CTA has warps are split over pivot-block and update-row
    CTAs (host_structure.cpp PlanSolveSplit); the split tasks, replayed in task order, solve every
    front as dense triangular solves do, and every wait is on an earlier task (no deadlock).  The
    tree order holds too: a front's forward tasks come after its children's, its backward tasks
    after its parent's.  (8, 4) is the device's split; the smaller ones split the small fronts."""
    p = synth.bundle_adjustment(num_cameras=80, num_points=2000, num_observations=8000, seed=5)
    c = p.to_c()
    assert shim.shim_build(C.byref(c)) == 0 and shim.shim_build_schur() == 0
    tile = 16
    tasks, npiv, ntiles, parent, w, m, cptr, clist = _factor_plan(shim, 1, tile)
    ns = len(npiv)
    out = _arr(2, np.int64)
    shim.shim_solve_split(warps, block_tiles, _ptr(out))
    nf, ntot = int(out[0]), int(out[1])
    kp, ku = _arr(ns, np.int32), _arr(ns, np.int32)
    tf, tsub = _arr(max(ntot, 1), np.int32), _arr(max(ntot, 1), np.int32)
    shim.shim_solve_split_arrays(*(_ptr(a) for a in (kp, ku, tf, tsub)))
    split = [s for s in range(ns) if npiv[s] + 0 > 0 and ntiles[s] > warps]
    assert [s for s in range(ns) if kp[s] > 0] == split
    assert len(split) > 0 and ntot > 0
    for s in split:
        assert kp[s] == -(-int(npiv[s]) // block_tiles)
        assert ku[s] == -(-(int(ntiles[s]) - int(npiv[s])) // block_tiles)
    first_fwd = {int(s): i for i, s in reversed(list(enumerate(tf[:nf])))}
    last_fwd = {int(s): i for i, s in enumerate(tf[:nf])}
    first_bwd = {int(s): nf + i for i, s in reversed(list(enumerate(tf[nf:ntot])))}
    last_bwd = {int(s): nf + i for i, s in enumerate(tf[nf:ntot])}
    for s in range(ns):
        for q in range(cptr[s], cptr[s + 1]):
            assert last_fwd[int(clist[q])] < first_fwd[s]
        if parent[s] >= 0:
            assert last_bwd[int(parent[s])] < first_bwd[s]
    fronts = [(int(w[s]), int(m[s])) for s in range(ns)]
    _replay_split_solve(fronts, kp, ku, tf[:ntot], tsub[:ntot], nf, block_tiles, tile, np.random.default_rng(11))
