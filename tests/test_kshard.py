"""k-sharded SCF host logic on CPU: two gloo ranks, each computing half of the k points with an
oracle-backed worker, must give the same P_new, step and energies as one rank with all k."""
import os

import numpy as np
import pytest

from oracle import forge_oracle as fo

M, NUMK, NU = 2, 3, 2.0


class OracleWorker:
    """The oracle restatement behind the k-shard worker interface (test only)."""

    def __init__(self, s, P, V, E_in):
        self.s = s
        self.g = fo.build_geometry(s)
        self.T = fo.pair_tables(s, self.g, use_c=False)
        self.LR = fo.long_range_interaction(s, self.g, use_c=False)
        self.P, self.V, self.E_in = P, V, E_in
        self.Nk, self.numb, self.N = s.Nk, s.numb, s.ndim

    def solve_local(self, k0, k1):
        s, g = self.s, self.g
        self.k0, self.k1 = k0, k1
        self.evecs, bands = {}, np.zeros((s.numb, k1 - k0))
        self.bulk = np.zeros((4, s.ndim, s.ndim), complex)
        for k in range(k0, k1):
            H = fo.hamiltonian(s, g, self.T, self.V, self.P, g.vk(k))
            w, Z = fo.eigh_lower(H, s.nUpper)
            bands[:, k - k0] = w[s.nLower - 1:]
            self.evecs[k] = Z[:, s.nLower - 1:]
            occ = np.conj(Z[:, :s.nLower - 1])
            Ck = occ @ np.conj(occ).T
            ivk1, ivk2 = (int(x) for x in g.kcomp[k])
            for c in range(4):
                self.bulk[c] += Ck * fo.bloch_phase_int(ivk1, ivk2, int(g.ucell1[c]), int(g.ucell2[c]), s.numk)
        return bands

    def set_global_bands(self, bands):
        self.bands = np.asarray(bands)

    def fermi(self):
        s = self.s
        se, idx, moms, _, band, kidx = fo.sort_energies_1spin(s, self.g, self.bands)
        self.sorted = (idx, moms, band, kidx)
        self.fl = fo.fermi_level(s, se)
        return self.fl

    def project_local(self):
        s, g = self.s, self.g
        nF, EF, nocc, npart, degf = self.fl
        idx, moms, band, kidx = self.sorted
        P = self.bulk.copy()
        zdeg = fo.zdeg_weight(s, degf)
        for q in range(nocc):
            k = int(kidx[q])
            if not (self.k0 <= k < self.k1):
                continue
            w = 1.0 if q < nocc - npart else zdeg
            zp = np.conj(self.evecs[k][:, band[q]])
            outer = np.outer(zp, np.conj(zp))
            ivk1, ivk2 = (int(x) for x in moms[q])
            for c in range(4):
                P[c] += outer * w * fo.bloch_phase_int(ivk1, ivk2, int(g.ucell1[c]), int(g.ucell2[c]), s.numk)
        return np.moveaxis(P / s.Nk, 0, 2)

    def step_and_mix(self, P_new, E_in):
        s = self.s
        Pn = np.moveaxis(P_new, 2, 0)
        dens = np.real(np.diagonal(self.P[0]))
        dn_new = np.real(np.diagonal(Pn[0]))
        step, E, _, _ = fo.optimal_step(s, self.T, self.LR, Pn, self.P, dn_new, dens, E_in)
        return step, E, Pn


def _initial(s):
    g = fo.build_geometry(s)
    T = fo.pair_tables(s, g, use_c=False)
    LR = fo.long_range_interaction(s, g, use_c=False)
    P, _ = fo.plain_guess(s, g, T)
    dens = np.real(np.diagonal(P[0]))
    return P, fo.potential(s, LR, dens), fo.energies(s, T, LR, P, dens)


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    from forge_gb300 import kshard
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    s = fo.Setup(ntheta=M, numk=NUMK, nfilling=NU)
    P, V, E = _initial(s)
    w = OracleWorker(s, P, V, E)
    step, E2, Pn = kshard.sharded_iteration(w, kshard.TorchComm(dist), E)
    if rank == 0:
        np.savez(out, Pn=Pn, step=step, E=[E2.kinetic, E2.fock, E2.hartree, E2.hubbard])
    dist.barrier()
    dist.destroy_process_group()


def test_partition_balanced():
    from forge_gb300.kshard import partition
    for Nk, world in ((16, 1), (16, 3), (144, 8), (5, 8)):
        parts = partition(Nk, world)
        assert parts[0][0] == 0 and parts[-1][1] == Nk
        sizes = [b - a for a, b in parts]
        assert max(sizes) - min(sizes) <= 1
        assert all(parts[i][1] == parts[i + 1][0] for i in range(world - 1))


def test_two_gloo_ranks_match_single_rank(tmp_path):
    import socket

    import torch.multiprocessing as mp
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    out = str(tmp_path / "r0.npz")
    mp.start_processes(_rank_main, args=(2, port, out), nprocs=2, start_method="spawn", join=True)
    got = np.load(out)
    # single rank, all k
    s = fo.Setup(ntheta=M, numk=NUMK, nfilling=NU)
    P, V, E = _initial(s)
    w = OracleWorker(s, P, V, E)
    w.solve_local(0, s.Nk)
    w.set_global_bands(w.solve_local(0, s.Nk))
    w.fermi()
    Pn = w.project_local()
    step, E2, _ = w.step_and_mix(Pn, E)
    assert np.max(np.abs(got["Pn"] - np.moveaxis(Pn, 2, 0))) <= 1e-12
    assert abs(float(got["step"]) - step) <= 1e-10
    assert np.allclose(got["E"], [E2.kinetic, E2.fock, E2.hartree, E2.hubbard], atol=1e-9)
