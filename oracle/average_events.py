"""CPU restatement of the reference's event averaging of the HBT files
(ebe_scripts/average_event_HBT_correlation_function.py): for every HBT* file
of the first UrQMD* folder's UrQMD_results, the element-wise mean over all
UrQMD* folders (glob order), written with numpy.savetxt(fmt='%.10e',
delimiter='  ').

Test and baseline infrastructure only (the timed CPU baseline of bench.py's
averaging leg); the product is hbt_host_average_events.
"""
from glob import glob
from os import makedirs, path

import numpy as np


def average_events(working_folder: str, avg_folder: str) -> int:
    makedirs(avg_folder, exist_ok=True)
    folders = glob(path.join(working_folder, "UrQMD*"))
    sub = "UrQMD_results"
    files = [f.split("/")[-1] for f in glob(path.join(folders[0], sub, "HBT*"))]
    nev = len(folders)
    for name in files:
        acc = 0.0 * np.loadtxt(path.join(folders[0], sub, name))
        for folder in folders:
            acc += np.loadtxt(path.join(folder, sub, name))
        np.savetxt(path.join(avg_folder, name), acc / nev, fmt="%.10e", delimiter="  ")
    return len(files)
