"""Stand-in for platformdirs (only the demo-data downloader imports it)."""


def user_cache_dir(*a, **k):
    return "/tmp"
