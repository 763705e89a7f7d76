// handle_table.cpp - HandleTable of the C++ facade.
//
// Growth follows src/CadR/HandleTable.cpp:113-337: the first handle creates
// one last-level table (handles 1..2047, entry 0 stays 0); handle 2048
// adds a routing table whose entries 0 and 1 point at last-level tables 0
// and 1 (two levels); every further 2,048 handles add a last-level table;
// handle 2048^2 adds a level-2 root whose entry 0 is the old routing table
// and entry 1 a new routing table (three levels).  Last-level table k always
// holds handles [k*2048, k*2048 + 2047], so
//   level 2: root[h >> 11][h & 0x7ff]
//   level 3: root[h >> 22][(h >> 11) & 0x7ff][h & 0x7ff]
// Every table is a 16 KiB allocation of the DataStorage; its host copy is
// uploaded by the next executeCopyOperations when it changed.
#include <CadR/DataStorage.h>

namespace CadR {

HandleTable::~HandleTable() { destroyAll(); }

// Frees every table's memory and forgets every handle (HandleTable.h:102,
// HandleTable.cpp:85); the storage calls it before its memory is released.
void HandleTable::destroyAll() noexcept
{
    for (auto& t : _tables)
        if (t->record) _storage->free(t->record);
    _tables.clear();
    _root = nullptr;
    _llt.clear();
    _l1.clear();
    _level = 0;
    _highest = 0;
}

HandleTable::Table* HandleTable::newTable()
{
    auto t = std::make_unique<Table>();
    t->record = _storage->alloc(numHandlesPerTable * sizeof(uint64_t));
    Table* p = t.get();
    _tables.push_back(std::move(t));
    return p;
}

void HandleTable::setEntry(Table* t, unsigned index, uint64_t value)
{
    t->addr[index] = value;
    t->dirty = true;
}

uint64_t HandleTable::create()
{
    if (_level == 0) {
        Table* llt = newTable();
        _llt.push_back(llt);
        _root = llt;
        _level = 1;
        _highest = 1;
        return _highest;
    }
    if (_level == 1) {
        if (_highest != handleBitsLevelMask) return ++_highest;
        Table* l1 = newTable();
        Table* llt = newTable();
        setEntry(l1, 0, _llt[0]->record->deviceAddress);
        setEntry(l1, 1, llt->record->deviceAddress);
        _llt.push_back(llt);
        _root = l1;
        _level = 2;
        return ++_highest;
    }
    if ((_highest & handleBitsLevelMask) != handleBitsLevelMask) return ++_highest;
    Table* llt = newTable();
    _llt.push_back(llt);
    if (_level == 2) {
        const unsigned l1Index = unsigned(_highest >> handleBitsLevelShift) + 1;
        if (l1Index < numHandlesPerTable) {
            setEntry(_root, l1Index, llt->record->deviceAddress);
            return ++_highest;
        }
        // two levels -> three levels
        Table* l1 = newTable();
        Table* l2 = newTable();
        setEntry(l1, 0, llt->record->deviceAddress);
        setEntry(l2, 0, _root->record->deviceAddress);
        setEntry(l2, 1, l1->record->deviceAddress);
        _l1.push_back(_root);
        _l1.push_back(l1);
        _root = l2;
        _level = 3;
        return ++_highest;
    }
    const unsigned l1Index = unsigned((_highest >> handleBitsLevelShift) & handleBitsLevelMask) + 1;
    if (l1Index < numHandlesPerTable) {
        const unsigned l2Index = unsigned(_highest >> (2 * handleBitsLevelShift));
        setEntry(_l1[l2Index], l1Index, llt->record->deviceAddress);
        return ++_highest;
    }
    Table* l1 = newTable();
    setEntry(l1, 0, llt->record->deviceAddress);
    const unsigned l2Index = unsigned(_highest >> (2 * handleBitsLevelShift)) + 1;
    setEntry(_root, l2Index, l1->record->deviceAddress);
    _l1.push_back(l1);
    return ++_highest;
}

void HandleTable::set(uint64_t handle, uint64_t addr)
{
    if (handle == 0 || handle > _highest) throw LogicError("HandleTable::set(): invalid handle");
    setEntry(_llt[handle >> handleBitsLevelShift], unsigned(handle & handleBitsLevelMask), addr);
}

uint64_t HandleTable::rootTableDeviceAddress() const { return _root ? _root->record->deviceAddress : 0; }

void HandleTable::uploadDirty()
{
    for (auto& t : _tables) {
        if (!t->dirty) continue;
        _storage->backend().upload(t->record->deviceAddress, t->addr.data(), sizeof(uint64_t) * numHandlesPerTable);
        t->dirty = false;
    }
}

}  // namespace CadR
