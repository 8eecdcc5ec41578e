// Link-time stand-ins for the preprocess dataset loaders (test infrastructure).
// preprocess_dataset.cpp is compiled only for generateGridStats; its main() is renamed
// by the recipe and never runs, so these loaders are never called.
#include "DatasetLoaderFactory.h"

std::unique_ptr<IDatasetLoader> DatasetLoaderFactory::create(DatasetType) { return nullptr; }
std::unique_ptr<IDatasetLoader> DatasetLoaderFactory::createFromPath(const std::string&) { return nullptr; }
