"""Console progress bar with dompap's call signature (dompap/tools/progress_bar.py)."""


def progress_bar(step: int, total: int, stride: int = 1, finalize: bool = False, width: int = 40) -> None:
    frac = 1.0 if finalize or total <= 0 else min(1.0, step / total)
    filled = int(width * frac)
    end = "\n" if finalize else "\r"
    print(f"[{'#' * filled}{'.' * (width - filled)}] {100 * frac:5.1f}%", end=end, flush=True)
