"""Simulation box information (``Sim_info.py:1-179`` of the reference).

Box sizes in cMpc/h for the simulations the reference knows, the half box
``L_0p5``, the output group ``snap_group`` ('Snapshot_<n>/' or '') and, with
``file_info=True``, where a simulation's group catalogue and snapshot files
are and how many there are (``Sim_info.py:136-176``).
"""

from __future__ import annotations

_TABLE = {
    "TNG100": (75.0, 0.6774),
    "TNG100_2": (75.0, 0.6774),
    "TNG300": (205.0, 0.6774),
    "EAGLE": (100.0 * 0.6777, 0.6777),
    "HorizonAGN": (100.0, 0.704),
}


# files per group catalogue / snapshot of the multi-file simulations
_FILES = {"TNG100": 448, "TNG100_2": 56, "TNG300": 600}
_EAGLE_Z = {"28": "z000p000", "17": "z001p487", "19": "z001p004", "21": "z000p736", "23": "z000p503",
            "25": "z000p271"}


class SimInfo:
    def __init__(self, sim_name, snapshot, boxsize=None, h=None, file_info=False):
        self.simname = sim_name
        self.N_files = None
        self.fof_folder = None
        self.snap_folder = None
        if snapshot is None:
            self.snapshot = None
            self.snap_group = ""
        else:
            self.snapshot = str(snapshot)
            self.snap_group = f"Snapshot_{self.snapshot}/"
        if isinstance(sim_name, str):
            self._specs()
            if file_info:
                self.get_file_info()
        else:
            self.boxsize = boxsize
            self.h = h
            self.L_0p5 = None if boxsize is None else boxsize / 2.0

    def _specs(self):
        name = self.simname
        if name in _TABLE:
            self.boxsize, self.h = _TABLE[name]
        elif "FLAMINGO" in name:
            if "L1" in name:
                self.boxsize = 1000.0 * 0.681
            elif "L2p8" in name:
                self.boxsize = 2800.0 * 0.681
            else:
                raise KeyError("Add an L1 or L2p8 suffix to your simname to specify which boxsize is used")
            self.h = 0.681
        elif "COLIBRE" in name:
            if "L4" in name:
                self.boxsize = 400.0 * 0.681
            elif "L2" in name:
                self.boxsize = 200.0 * 0.681
            else:
                raise KeyError("Add an L4 or L2 suffix to your simname to specify which boxsize is used")
            self.h = 0.681
        else:
            raise KeyError(
                "Simulation name not recognised. Choose from [TNG100, TNG100_2, TNG300, EAGLE, HorizonAGN, "
                "FLAMINGO_L1, FLAMINGO_L2p8, COLIBRE_L400, COLIBRE_L200].")
        self.L_0p5 = self.boxsize / 2.0

    def get_specs(self):
        """Box size and h of a named simulation (Sim_info.py:83-135)."""
        self._specs()

    def get_file_info(self):
        """Group catalogue and snapshot file stems and file counts."""
        name, snap = self.simname, self.snapshot
        if name in _FILES:
            self.fof_folder = f"/fof_subhalo_tab_0{snap}/fof_subhalo_tab_0{snap}"
            self.snap_folder = f"/snap_0{snap}/snap_0{snap}"
            self.N_files = _FILES[name]
        elif name == "EAGLE":
            z = _EAGLE_Z[snap]
            self.snap_folder = f"/snap_0{snap}/RefL0100N1504/snapshot_0{snap}_{z}/snap_0{snap}_{z}"
            self.fof_folder = None
            self.N_files = 256
        elif name == "HorizonAGN":
            self.fof_folder = self.snap_folder = None
            self.N_files = 1.
        elif "FLAMINGO" in name or "COLIBRE" in name:
            self.fof_folder = self.snap_folder = None
            self.N_files = 1
        else:
            raise KeyError(
                "Simulation name not recognised. Choose from [TNG100, TNG300, EAGLE, HorizonAGN, FLAMINGO_L1_m8, "
                "FLAMINGO_L1_m9, FLAMINGO_L1_m10, FLAMINGO_L2p8_m9,, COLIBRE_L400, COLIBRE_L200].")
