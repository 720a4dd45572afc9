"""Console progress bar with dompap's call signature and marks
(dompap/tools/progress_bar.py:1-21)."""
from __future__ import annotations


def progress_bar(current_step, total_num_steps, this_stride, finalize=False) -> None:
    """Print progress for ``current_step`` of ``total_num_steps`` (called every
    ``this_stride`` steps): a new line with the time and the step count every
    50 strides, ``|`` every 10, ``:`` every 5, ``.`` otherwise, then the
    percentage done, which the next call overwrites; ``finalize`` replaces the
    percentage by ``done`` and ends the line."""
    from datetime import datetime

    back = "\b" * 7  # erase the previous percentage
    if finalize:
        print(back + "  done")
        return
    parts = [back]
    if current_step % (this_stride * 50) == 0:
        parts.append(f"{'|' + chr(10) if current_step > 0 else ''}{datetime.now()} {current_step:12,} ")
    if current_step % (this_stride * 10) == 0:
        parts.append("|")
    elif current_step % this_stride == 0:
        parts.append(":" if current_step % (this_stride * 5) == 0 else ".")
    parts.append(f" {current_step / total_num_steps * 100:5.1f}%")
    print("".join(parts), end="", flush=True)
